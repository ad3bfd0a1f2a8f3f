// Whole CLOUD models on the device, one per CTA, and the kernels of the C ABI.
//
//   model set-up      physics-core.f90:42-73, cloud.f90:20-31, chemistry.f90:46-141
//   interval loop     wrap.f90:657-690 with cloud.f90:39-51 (updateTargetTime)
//   updateChemistry   chemistry.f90:145-239 (retries, stall detector)
//   integrateODESystem chemistry.f90:241-292 (abstol vector, ISTATE recovery)
//   output rows       io.f90:74-82
//   collapse physics  collapse.f90:27-115 (initializePhysics, updateTargetTime,
//                     updatePhysics), in place of cloud.f90's when
//                     ucl_model_params::collapse is 1-4
//   hot-core physics  hotcore.f90:22-79 when ucl_model_params::hotcore is 1-6
#pragma once
#include "ucl_bdf.cuh"
#include "ucl_collapse.cuh"
#include "ucl_hotcore.cuh"

namespace ucl {

// updateTargetTime (cloud.f90:39-51).  floor(log10 t) is taken exactly (by
// comparison with exact powers of ten) so a power-of-ten time is never
// misplaced by the rounding of log10.
__device__ double target_time(double ty, double spy) {
  if (ty >= 1.0e6) return (ty + 1.0e5) * spy;
  if (ty > 10.0) {
    int k = (int)floor(log10(ty));
    auto p10 = [](int e) { double p = 1.0; for (int i = 0; i < e; ++i) p *= 10.0; return p; };
    if (k < 1) k = 1;
    if (k > 5) k = 5;  // 10 < ty < 1e6 here
    while (k < 5 && p10(k + 1) <= ty) ++k;
    while (k > 1 && p10(k) > ty) --k;
    const double om = p10(k);
    return ((floor(ty / om) + 1.0) * om) * spy;
  }
  if (ty > 0.0) return 10 * ty * spy;
  return spy * 1.0e-7;
}

// Inputs and outputs of a batched solve.  Per-model arrays use the strides
// of the context's largest network, so models of different networks can
// share one launch: model i's start vector is start[i*start_stride ...],
// its rows abund[(i*max_rows + r)*ab_stride ...] and
// rates[(i*max_rows + r)*rate_stride ...].
struct SolveIO {
  const ucl_model_params* params;
  const double* start;       // nullptr: elemental start of initializeChemistry
  double* phys;
  double* abund;
  double* rates;             // nullptr: no rates rows
  int* nrows;
  int* flags;
  ucl_model_stats* stats;    // may be nullptr
  int nmodels, max_rows, start_stride, ab_stride, rate_stride;
  const DevNet* nets;        // device array of the context's networks
  const int* net_of;         // network of each model (nullptr: all network 0)
};

// start-of-interval quantities of updateChemistry (chemistry.f90:166-200)
template <typename T>
__device__ void interval_start(Ctx<T>& C, bool refresh_density) {
  Shared& sh = *C.sh;
  const DevNet& N = *C.N;
  double* y = C.y;
  if (threadIdx.x == 0) {
    SysPhys& S = sh.S;
    if (refresh_density) y[N.neq - 1] = S.dens;
    S.h2col = 0.5 * y[N.nh2] * S.dens * S.cs;
    S.cocol = 0.5 * y[N.nco] * S.dens * S.cs;
    S.ccol = 0.5 * y[N.nc] * S.dens * S.cs;
    double sb = 0.0, ss = 0.0;
    for (int i = 0; i < N.n_bulk; i++) sb = i == 0 ? y[N.bulk_list[i]] : sb + y[N.bulk_list[i]];
    for (int i = 0; i < N.n_surface; i++) ss = i == 0 ? y[N.surface_list[i]] : ss + y[N.surface_list[i]];
    // (a network without ices has no SURFACE/BULK totals: its nsurf/nbulk
    // name the density slot, which must not be overwritten)
    if (N.n_bulk > 0) y[N.nbulk] = sb;
    if (N.n_surface > 0) y[N.nsurf] = ss;
    S.sm = fmax(1e-30, ss);
    S.sb = fmax(1e-30, sb);
    if (N.n_refr > 0) {  // refractory ices do not count as bulk (chemistry.f90:196)
      double r = 0.0;
      for (int i = 0; i < N.n_refr; i++) r += y[N.refr_list[i]];
      S.sb = S.sb - r;
    }
    const double q = cK.NUM_SITES_PER_GRAIN / (cK.GAS_DUST_DENSITY_RATIO * S.sb);
    S.blr = q < 1.0 ? q : 1.0;
    photo_setup(S, sh.P.radfield);
  }
  __syncthreads();
}

// x**k for an integer k >= 0 by the right-to-left binary method (Knuth,
// TAOCP 4.6.3): square x while halving k, multiplying the squares of the set
// bits into the result, the way compiled Fortran evaluates a real raised to
// a variable integer power.
__device__ __forceinline__ double ipow_bin(double x, int k) {
  unsigned e = (unsigned)k;
  double r = (e & 1u) ? x : 1.0;
  while (e >>= 1) {
    x = x * x;
    if (e & 1u) r = r * x;
  }
  return r;
}

// H2 cosmic-ray dissociation rate of ionizationDependency
// (physics-core.f90:121-157): 10^(sum_k c_k log10(N)^k) * zeta, with N the
// parcel's column density and c_k the L or H model coefficients of
// physics-core.f90:29-37 (Padovani et al. 2018b fits; data).
__device__ double h2_crp_rate(const ucl_model_params& P, double coldens) {
  const double cL[10] = {1.582911005330e7, -6.465722684896e6, 1.172189025424e6, -1.237950798073e5,
                         8.393404654312e3, -3.788811358130e2, 1.138688455029e1,  -2.197136304567e-1,
                         2.469841278950e-3, -1.232393620924e-5};
  const double cH[10] = {1.217227462831e7, -4.989649250304e6, 9.079152156645e5, -9.624890825395e4,
                         6.551161486120e3, -2.968976216187e2, 8.959037875226e0,  -1.735757324445e-1,
                         1.959267277734e-3, -9.816996707980e-6};
  const double* c = P.ionModel == 'H' ? cH : cL;
  const double x = log10(coldens);
  double s = 0.0;
  for (int k = 0; k < 10; ++k) s = s + c[k] * ipow_bin(x, k);
  return pow(10.0, s) * P.zeta;
}

// One output row (io.f90:74-93).  With rates_out, the row of the rates
// array too: the reference's rate() as it stands at output time, i.e. the
// interval's calculateReactionRates values with the H2 and CO
// photodissociation entries as the last F evaluation left them
// (chemistry.f90:315-318); all zero before the first interval.
template <typename T>
__device__ void write_row(Ctx<T>& C, const SolveIO& io, int mi) {
  Shared& sh = *C.sh;
  const DevNet& N = *C.N;
  const int nspec = N.nspec, max_rows = io.max_rows;
  const int row = sh.ms.row;
  double* ab = io.abund + ((size_t)mi * max_rows + row) * io.ab_stride;
  for (int i = threadIdx.x; i < nspec; i += NT) ab[i] = C.y[i];
  if (io.rates) {
    double* rr = io.rates + ((size_t)mi * max_rows + row) * io.rate_stride;
    for (int j = threadIdx.x; j < N.nreac; j += NT) {
      double v = 0.0;
      if (row > 0) v = j == N.rx_h2hv ? sh.R.kh2 : j == N.rx_cohv ? sh.R.kco : C.W.rate[j];
      rr[j] = v;
    }
  }
  if (threadIdx.x == 0) {
    double* ph = io.phys + ((size_t)mi * max_rows + row) * UCL_N_PHYS;
    ph[0] = sh.ms.tyears;
    ph[1] = sh.S.dens;
    ph[2] = sh.S.T;
    ph[3] = sh.S.Td;
    ph[4] = sh.S.av;
    ph[5] = sh.P.radfield;
    ph[6] = sh.P.zeta;
    ph[7] = 1.0;
    sh.ms.row = row + 1;
  }
  __syncthreads();
}

// initializePhysics of the collapse module, the part after the mode checks
// (collapse.f90:56-57): density = rhofit(rin, ...) at t = 0 and, for the
// Bonnor-Ebert modes, the mass inside the parcel (findMassInRadius,
// 1000-step trapezoid).  All threads call.  (The collapse functions are not
// inlined, so they leave the register allocation of the solver alone.)
template <typename T>
__device__ __noinline__ void collapse_init(Ctx<T>& C) {
  Shared& sh = *C.sh;
  ModelState& ms = sh.ms;
  const int cm = ms.cmode;
  const double rho0 = col_rho0fit(cm, 0.0, ms.ctmax), r0 = col_r0fit(cm, 0.0, ms.ctmax), a = col_afit(cm, 0.0);
  double mass = 0.0;
  if (cm <= 2) mass = col_trapezoid(1, cm, 1000, 0.0, ms.crad / 1000, rho0, r0, a, sh.red);
  if (threadIdx.x == 0) {
    sh.S.dens = col_rhofit(cm, sh.P.rin, rho0, r0, a);
    ms.cmass = mass;
  }
  __syncthreads();
}

// updatePhysics of the collapse module (collapse.f90:76-106) after
// coreUpdatePhysics: the column density to the cloud edge from the current
// profile (findcoldens, 1e4-step trapezoid), Av from it, the parcel's new
// radius and its density.  All threads call.
template <typename T>
__device__ __noinline__ void collapse_update(Ctx<T>& C) {
  Shared& sh = *C.sh;
  ModelState& ms = sh.ms;
  const ucl_model_params& P = sh.P;
  const int cm = ms.cmode;
  const double t = ms.tyears;
  const double rho0 = col_rho0fit(cm, t, ms.ctmax), r0 = col_r0fit(cm, t, ms.ctmax), a = col_afit(cm, t);
  const double size = P.rout - P.rin;
  double coldens = 0.0;
  if (size > 0.0) coldens = col_trapezoid(0, cm, 10000, P.rin, size / 10000, rho0, r0, a, sh.red);
  double rad = ms.crad;
  __shared__ int s_err;
  if (threadIdx.x == 0) s_err = 0;
  __syncthreads();
  if (cm <= 2) {
    // the radius enclosing the parcel's initial mass (findNewRadius with r = rout)
    rad = col_new_radius(cm, ms.cmass, P.rout, rho0, r0, a, reinterpret_cast<double*>(C.lu_smem), &s_err);
  } else if (threadIdx.x == 0) {
    // dt = targetTime - currentTime: zero once the chemistry has reached targetTime
    const double dt = ms.target - ms.t;
    const double drad = col_vrfit(cm, ms.crad, col_rminfit(cm, t), col_vminfit(cm, t), col_avfit(cm, t)) * dt / cK.PC;
    rad = ms.crad + drad;
  }
  if (threadIdx.x == 0) {
    ms.coldens = coldens;
    sh.S.av = P.baseAv + coldens / 1.6e21;
    if (s_err || !(rad >= 0.0)) ms.flag = UCL_INT_UNRECOVERABLE_ERROR;
    ms.crad = rad;
    sh.S.dens = col_rhofit(cm, rad, rho0, r0, a);
  }
  __syncthreads();
}

template <typename T>
__device__ void run_model(Ctx<T>& C, const SolveIO& io, int mi, const ucl_model_params* params) {
  const int max_rows = io.max_rows;
  Shared& sh = *C.sh;
  ModelState& ms = sh.ms;
  SysPhys& S = sh.S;
  const DevNet& N = *C.N;
  const int tid = threadIdx.x, n = C.n;
  double* y = C.y;
  if (tid == 0) {
    sh.P = params[mi];
    const ucl_model_params& P = sh.P;
    ms.t0 = globaltimer_ns();
    const double cloudSize = (P.rout - P.rin) * cK.PC;
    S.cs = cloudSize / (double)(float)P.points;
    S.T = P.initialTemp;
    S.Td = S.T;
    ms.coldens = (double)(float)P.points * cloudSize / (double)(float)P.points * P.initialDens;
    S.av = P.baseAv + ms.coldens / 1.6e21;
    S.dens = P.freefall ? (double)1.001f * P.initialDens : P.initialDens;
    S.phi = P.phi;
    S.h2crp = 0.0;  // h2CRPRate before the first physics update: a fresh process's zero
    ms.t = 0.0;
    ms.tyears = 0.0;
    ms.flag = 0;
    ms.row = 0;
    ms.fail_count = 0;
    ms.retries = 0;
    ms.abstol_factor = P.abstol_factor;
    ms.nst = ms.nfe = ms.nje = ms.nlu = ms.nni = ms.ncfn = ms.netf = 0;
    for (int k = 0; k < 5; k++) ms.tacc[k] = 0;
    sh.d.mxstep = P.mxstep;
    // coreInitializePhysics's checks (physics-core.f90:55-64) give
    // PHYSICS_INIT_ERROR; so does points > 1: coreUpdatePhysics reads
    // coldens(dstep-1) = coldens(0), outside coldens(1:points), for the first
    // parcel (physics-core.f90:80), so the reference's multi-parcel result is
    // undefined and the parcels share one retried targetTime
    if (P.points != 1 || (P.ionModel != 'L' && P.ionModel != 'H') ||
        (P.improvedH2CRPDissociation && !P.cosmicRayAttenuation))
      ms.flag = UCL_PHYSICS_INIT_ERROR;
    // collapse module set-up (collapse.f90:27-58): maxTime and finalTime of
    // the Bonnor-Ebert modes, the parcel at rout; another mode number is
    // "unacceptable collapse mode"
    ms.cmode = P.collapse;
    ms.ctmax = 0.0;
    ms.cmass = 0.0;
    if (P.collapse != 0) {
      if (P.collapse < 1 || P.collapse > 4) ms.flag = UCL_PHYSICS_INIT_ERROR;
      if (P.collapse == 1) ms.ctmax = 1.175e6;
      if (P.collapse == 2) ms.ctmax = 1.855e5;
      if (P.collapse == 1 || P.collapse == 2) sh.P.finalTime = (double)0.97f * ms.ctmax;
      ms.crad = 1 * P.rout / (double)(float)P.points;
    }
    // hot-core module set-up (hotcore.f90:22-45): temp_indx beyond the six
    // masses is an error; the reference does not check below 1, which would
    // index outside its tables, so that is rejected too, as is a model with
    // both modules
    ms.hmode = P.hotcore;
    if (P.hotcore != 0 && (P.hotcore < 1 || P.hotcore > 6 || P.collapse != 0)) ms.flag = UCL_PHYSICS_INIT_ERROR;
  }
  __syncthreads();
  const ucl_model_params& P = sh.P;
  if (ms.cmode != 0 && ms.flag == 0) collapse_init(C);
  // initial abundances (initializeChemistry, chemistry.f90:57-105)
  for (int i = tid; i < n; i += NT) y[i] = 1.0e-30;
  __syncthreads();
  if (io.start) {
    for (int i = tid; i < n; i += NT) y[i] = io.start[(size_t)mi * io.start_stride + i];
  } else {
    if (tid == 0) {
      y[N.no] = P.fo; y[N.nn] = P.fn; y[N.nmg] = P.fmg; y[N.np] = P.fp; y[N.nf] = P.ff;
      y[N.nna] = P.fna; y[N.nli] = P.fli; y[N.npah] = P.fpah;
      y[N.nsx] = P.fs; y[N.nsix] = P.fsi; y[N.nclx] = P.fcl;
      if (P.ion == 0) { y[N.nc] = P.fc; y[N.ncx] = 1.e-10; }
      else if (P.ion == 1) { y[N.nc] = P.fc * 0.5; y[N.ncx] = P.fc * 0.5; }
      else if (P.ion == 2) { y[N.nc] = 1.e-10; y[N.ncx] = P.fc; }
      y[N.n18o] = P.f18o; y[N.n15n] = P.f15n; y[N.n13c] = P.f13c;
      y[N.nelec] = y[N.ncx] + y[N.nsix] + y[N.nsx] + y[N.nclx] + y[N.nmgx];
    }
    __syncthreads();
    for (int i = tid; i < n; i += NT) y[i] = y[i] * P.metallicity;
    __syncthreads();
    if (tid == 0) {
      y[N.nh] = P.fh;
      y[N.nh2] = 0.5 * (1.0 - P.fh);
      y[N.nd] = P.fd;
      y[N.nhe] = P.fhe;
      y[n - 1] = S.dens;
    }
  }
  __syncthreads();
  if (ms.flag == 0) write_row(C, io, mi);
  for (;;) {
    if (tid == 0)
      ms.go = (ms.flag == 0) && ((P.endAtFinalDensity && S.dens < P.finalDens) ||
                                 (!P.endAtFinalDensity && ms.tyears < P.finalTime));
    __syncthreads();
    if (!ms.go) break;
    if (tid == 0) {
      const double told = ms.t;
      ms.tyears = ms.t / cK.SECONDS_PER_YEAR;
      ms.target = ms.cmode   ? col_target_time(ms.tyears, cK.SECONDS_PER_YEAR)
                  : ms.hmode ? hc_target_time(ms.tyears, cK.SECONDS_PER_YEAR)
                             : target_time(ms.tyears, cK.SECONDS_PER_YEAR);
      ms.t = told;
      ms.loop = 0;
      ms.orig = ms.target;
    }
    __syncthreads();
    // updateChemistry
    for (;;) {
      if (tid == 0) ms.go = (ms.t < ms.target) && (ms.loop < 10);
      __syncthreads();
      if (!ms.go) break;
      interval_start(C, !P.freefall);
      ph_begin(ms);
      dev_rates(N, P, S, y, C.W.rate, C.aux);
      ph_end(ms, PH_RATES);
      for (int i = tid; i < n; i += NT) {
        double a = ms.abstol_factor * y[i];
        if (a < P.abstol_min) a = P.abstol_min;
        C.atol[i] = a;
      }
      __syncthreads();
      const int istate = dv_ode<T>(C, ms.target, P.reltol);
      if (tid == 0) {
        DvState& d = sh.d;
        ms.nst += d.nst; ms.nfe += d.nfe; ms.nje += d.nje; ms.nlu += d.nlu;
        ms.nni += d.nni; ms.ncfn += d.ncfn; ms.netf += d.netf;
        if (istate == -1 || istate == -4 || istate == -5)
          ms.target = ms.t + (ms.target - ms.t) * (double)0.1f;
        else if (istate == -2)
          ms.abstol_factor = ms.abstol_factor * 10.0;
        else if (istate == -3)
          ms.flag = UCL_INT_UNRECOVERABLE_ERROR;
      }
      __syncthreads();
      if (ms.flag < 0) break;
      if (P.enforceChargeConservation && tid == 0) {
        // electrons = sum of the positive ions after every DVODE call
        // (integrateODESystem, chemistry.f90:287-291)
        double e = 0.0;
        for (int k = 0; k < N.n_ion; ++k) e += y[N.ion_list[k]];
        if (N.n_ion > 0) y[N.nelec] = e;
      }
      __syncthreads();
      for (int i = tid; i < n; i += NT)
        if (y[i] < 1.0e-30) y[i] = 1.0e-30;
      __syncthreads();
      if (tid == 0) {
        S.dens = y[n - 1];
        ms.loop++;
        if (ms.loop > 1) ms.retries++;
      }
      __syncthreads();
    }
    if (tid == 0 && ms.flag == 0) {
      if (ms.loop == 10) ms.flag = UCL_INT_TOO_MANY_FAILS_ERROR;
      if (fabs(ms.orig - ms.target) < (double)0.001f * ms.orig) ms.fail_count = 0;
      else ms.fail_count++;
      if (ms.fail_count > 10) ms.flag = UCL_INT_TOO_MANY_FAILS_ERROR;
      if (ms.flag == 0) {
        ms.tyears = ms.target / cK.SECONDS_PER_YEAR;
        ms.coldens = S.cs * S.dens;  // coreUpdatePhysics (physics-core.f90:75-88)
        S.av = P.baseAv + ms.coldens / 1.6e21;
        S.Td = S.T;
        if (P.cosmicRayAttenuation && P.improvedH2CRPDissociation) S.h2crp = h2_crp_rate(P, ms.coldens);
        if (ms.hmode) {  // the hot-core module's updatePhysics: the temperature ramp
          S.T = hc_temperature(ms.hmode, S.T, ms.t, P.initialTemp, P.maxTemperature, (P.rout - P.rin) * cK.PC,
                               P.rout, P.points);
          S.Td = S.T;
        }
        if (ms.row >= max_rows) ms.flag = UCL_NOT_ENOUGH_TIMEPOINTS_ERROR;
      }
    }
    __syncthreads();
    if (ms.flag < 0) break;
    if (ms.cmode != 0) {
      collapse_update(C);
      if (ms.flag < 0) break;
    }
    write_row(C, io, mi);
  }
  if (tid == 0) {
    io.nrows[mi] = ms.row;
    io.flags[mi] = ms.flag;
    if (io.stats) {
      ucl_model_stats st;
      st.nst = ms.nst; st.nfe = ms.nfe; st.nje = ms.nje; st.nlu = ms.nlu; st.nni = ms.nni;
      st.ncfn = ms.ncfn; st.netf = ms.netf;
      st.n_intervals = ms.row;
      st.n_retries = ms.retries;
      st.solve_ms = (double)(globaltimer_ns() - ms.t0) * 1e-6;
      st.t_rates_ms = ms.tacc[PH_RATES] * 1e-6;
      st.t_rhs_ms = ms.tacc[PH_RHS] * 1e-6;
      st.t_jac_ms = ms.tacc[PH_JAC] * 1e-6;
      st.t_lu_ms = ms.tacc[PH_LU] * 1e-6;
      st.t_solve_ms = ms.tacc[PH_SOLVE] * 1e-6;
      const unsigned long long t1 = globaltimer_ns();
      st.queue_ms = ms.t0 > ms.ta ? (double)(ms.t0 - ms.ta) * 1e-6 : 0.0;
      st.latency_ms = t1 > ms.ta ? (double)(t1 - ms.ta) * 1e-6 : 0.0;
      io.stats[mi] = st;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// shared-memory carve-up of the solver kernels
struct SmemLayout {
  size_t y, savf, acor, ewt, atol, tmp, wJ, wJi, yh, xs, xt, flux, part, dfa, dfb, vec, aux, lu, total;
};

template <typename T>
__host__ __device__ inline SmemLayout smem_layout(int n, int nreac, int nchunk) {
  SmemLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += (bytes + 15) / 16 * 16; return r; };
  L.y = take(8 * n); L.savf = take(8 * n); L.acor = take(8 * n); L.ewt = take(8 * n);
  L.atol = take(8 * n); L.tmp = take(8 * n); L.wJ = take(8 * n); L.wJi = take(8 * n);
  L.yh = take(8 * (size_t)LMAXP * n);
  L.xs = take(sizeof(T) * n); L.xt = take(sizeof(T) * n);
  const size_t u0 = o;
  // union: chemistry scratch | rates scratch | LU panel
  size_t oc = u0;
  auto takec = [&](size_t bytes) { size_t r = oc; oc += (bytes + 15) / 16 * 16; return r; };
  L.flux = takec(8 * (size_t)nreac);
  L.part = takec(8 * (size_t)nchunk);
  L.dfa = takec(8 * (size_t)nreac);
  L.dfb = takec(8 * (size_t)nreac);
  L.vec = takec(8 * (size_t)JAC_VEC_DOUBLES);
  L.aux = L.dfa;
  L.lu = u0;
  size_t lu_end = u0 + lu_smem_bytes<T>(n);
  L.total = oc > lu_end ? oc : lu_end;
  return L;
}

template <typename T>
__device__ Ctx<T> make_ctx(const DevNet* N, Shared* sh, char* smem, const SmemLayout& L, Slot<T> W) {
  Ctx<T> C;
  C.N = N; C.sh = sh; C.n = N->neq; C.W = W;
  C.y = (double*)(smem + L.y); C.savf = (double*)(smem + L.savf); C.acor = (double*)(smem + L.acor);
  C.ewt = (double*)(smem + L.ewt); C.atol = (double*)(smem + L.atol); C.tmp = (double*)(smem + L.tmp);
  C.wJ = (double*)(smem + L.wJ); C.wJi = (double*)(smem + L.wJi); C.xs = (T*)(smem + L.xs);
  C.xt = (T*)(smem + L.xt);
  C.flux = (double*)(smem + L.flux); C.part = (double*)(smem + L.part); C.dfa = (double*)(smem + L.dfa);
  C.dfb = (double*)(smem + L.dfb); C.vec = (double*)(smem + L.vec); C.aux = (double*)(smem + L.aux);
  C.lu_smem = smem + L.lu;
  C.W.yh = (double*)(smem + L.yh);
  return C;
}

// per-slot workspace in global memory, sized for the context's largest
// network (n = NEQ, nreac reactions)
template <typename T>
struct SlotArrays {
  double* yh;
  double* rate;
  T* J;
  T* P;
  int* perm;
  T* scr;
  T* dinv;
  double* jpart;
  double* ginv;
  int n, nreac, njch;
};

template <typename T>
__device__ __forceinline__ Slot<T> slot_of(const SlotArrays<T>& A, int s) {
  const int n = A.n, nreac = A.nreac;
  Slot<T> W;
  W.yh = nullptr;  // shared memory, set by make_ctx
  W.rate = A.rate + (size_t)s * nreac;
  W.J = A.J + (size_t)s * mat_stride(n);
  W.P = A.P + (size_t)s * mat_stride(n);
  W.perm = A.perm + (size_t)s * n;
  W.scr = A.scr + (size_t)s * 2 * LuCfg<T>::NB * n;
  W.dinv = A.dinv + (size_t)s * dinv_elems(n);
  W.jpart = A.jpart + (size_t)s * A.njch;
  W.ginv = A.ginv + (size_t)s * MAX_INV * MAX_INV;
  return W;
}

// bounded wait of the admission loop: at most this many sleeps of 20 us
constexpr unsigned ADMIT_SLEEP_LIMIT = 1u << 26;

// Admission order of a batch: longest-expected first, so that the slowest
// models do not start last and set the makespan.  The expected cost grows
// with density and temperature (faster grain-surface chemistry makes the
// system stiffer); the key is log10(n) + 0.05 T.  Results of each model do
// not depend on the order.  Batches above ORDER_MAX keep index order.
constexpr int ORDER_MAX = 4096;
__global__ void __launch_bounds__(1024) k_order(const ucl_model_params* params, int nmodels, int* order) {
  __shared__ float key[ORDER_MAX];
  __shared__ int idx[ORDER_MAX];
  const int tid = threadIdx.x;
  if (nmodels > ORDER_MAX) {
    for (int i = tid; i < nmodels; i += blockDim.x) order[i] = i;
    return;
  }
  int P = 1;
  while (P < nmodels) P <<= 1;
  for (int i = tid; i < P; i += blockDim.x) {
    if (i < nmodels) {
      key[i] = (float)(log10(params[i].initialDens) + 0.05 * params[i].initialTemp);
      idx[i] = i;
    } else {
      key[i] = -INFINITY;
      idx[i] = 0x7fffffff;
    }
  }
  __syncthreads();
  // bitonic sort into "before" order: larger key first, then smaller index
  auto before = [&](int a, int b) { return key[a] > key[b] || (key[a] == key[b] && idx[a] < idx[b]); };
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          if (up ? before(ixj, i) : before(i, ixj)) {
            const float tk = key[i]; key[i] = key[ixj]; key[ixj] = tk;
            const int ti = idx[i]; idx[i] = idx[ixj]; idx[ixj] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < nmodels; i += blockDim.x) order[i] = idx[i];
}

// Live request queue of the serving mode: a ring of `cap` records whose
// parameters and flags live in host-pinned memory mapped into the device's
// address space.  Request k (numbered from 0) uses record k % cap: its
// parameters are req[k % cap], its outputs the record's rows of the solve's
// output arrays.  The host publishes request k by writing req[k % cap] and
// then tail = k + 1 (release); it publishes request k only after it has
// taken the outputs of request k - cap, so a record is never overwritten
// while in use.  The device sets done[k % cap] = k + 1 (release, after the
// outputs are written).  closed = 1 ends the session once every published
// request is claimed.
struct LiveQueue {
  const ucl_model_params* req;  // [cap]
  const unsigned* tail;
  const unsigned* closed;
  unsigned* done;               // [cap]
  int* status;                  // set to UCL_E_TIMEOUT by a CTA whose wait gave up
  int cap;
  unsigned idle_limit;          // sleeps of 20 us an idle CTA waits for a request before it gives up
};

__device__ __forceinline__ unsigned ld_acquire_sys(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.sys.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(unsigned* p, unsigned v) {
  asm volatile("st.release.sys.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Persistent solver: each CTA pulls model indices from a device counter
// (requests in index order, or through `order` when given).  The launch
// epoch is the first CTA's start time.  With an arrival schedule (seconds
// after the epoch, ascending), a request is not started before its arrival;
// queue and latency times are measured from arrival (from the epoch without
// a schedule).  With a live queue (q.cap > 0) the counter numbers requests
// that the host appends while the kernel runs (LiveQueue).  A model's
// network tables are loaded into shared memory when it differs from the
// previous model's network.
template <typename T>
__global__ void __launch_bounds__(NT, 1) k_solve_models(SolveIO io, SlotArrays<T> ws, int* counter,
                                                     unsigned long long* epoch, const double* arrival_s,
                                                     const int* order, LiveQueue q) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Shared sh;
  __shared__ DevNet sN;
  __shared__ unsigned long long t_epoch;
  __shared__ unsigned req_no;
  const int nmodels = io.nmodels;
  if constexpr (sizeof(T) == 4) tc_setup(&sh.tc);
  if (threadIdx.x == 0) {
    const unsigned long long now = globaltimer_ns();
    const unsigned long long old = atomicCAS(epoch, 0ull, now);
    t_epoch = old ? old : now;
  }
  int cur_net = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const int k = atomicAdd(counter, 1);
      sh.ms.ta = t_epoch;
      if (q.cap > 0) {
        // wait (bounded) until request k is published or the session ends
        int mi = nmodels;
        unsigned it = 0;
        for (; it < q.idle_limit; ++it) {
          if ((unsigned)k < ld_acquire_sys(q.tail)) { mi = k % q.cap; break; }
          if (ld_acquire_sys(q.closed)) break;
          __nanosleep(20000);
        }
        if (it == q.idle_limit) atomicExch(q.status, UCL_E_TIMEOUT);
        sh.ms.ta = globaltimer_ns();
        req_no = (unsigned)k;
        sh.ms.model = mi;
      } else {
        sh.ms.model = (order && k < nmodels) ? order[k] : k;
        const int mi = sh.ms.model;
        if (mi < nmodels && arrival_s) {
          const double a = arrival_s[mi];
          const unsigned long long ta = t_epoch + (a > 0.0 ? (unsigned long long)(a * 1e9) : 0ull);
          sh.ms.ta = ta;
          for (unsigned it = 0; it < ADMIT_SLEEP_LIMIT && globaltimer_ns() < ta; ++it) __nanosleep(20000);
        }
      }
    }
    __syncthreads();
    const int mi = sh.ms.model;
    if (mi >= nmodels) break;
    const int kn = io.net_of ? io.net_of[mi] : 0;
    if (kn != cur_net) {
      // this model's network tables into shared memory
      for (int i = threadIdx.x; i < (int)(sizeof(DevNet) / sizeof(int)); i += NT)
        reinterpret_cast<int*>(&sN)[i] = reinterpret_cast<const int*>(io.nets + kn)[i];
      __syncthreads();
      cur_net = kn;
    }
    Ctx<T> C = make_ctx<T>(&sN, &sh, smem, smem_layout<T>(sN.neq, sN.nreac, sN.nchunk), slot_of(ws, blockIdx.x));
    run_model<T>(C, io, mi, q.cap > 0 ? q.req : io.params);
    if (q.cap > 0 && threadIdx.x == 0) {
      __threadfence_system();
      st_release_sys(q.done + mi, req_no + 1u);
    }
  }
  if constexpr (sizeof(T) == 4) tc_teardown(&sh.tc);
}

// Batched dense LU (ucl_lu_factor_device): one CTA per matrix, the same
// factorisation the solver applies to its Newton matrices.
template <typename T>
__global__ void __launch_bounds__(NT) k_lu_batch(T* mats, int n, int* perm, int* info, T* scr, int nsys,
                                                 int allow_tc = 1) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int si[LU_SI_INTS];
  __shared__ int lperm[MAX_NEQ];
  __shared__ TcState tc;
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const bool use_tc = allow_tc && LuSmem<T>::tc_ok(n);
  if (use_tc) tc_setup(&tc, tc_cols_for(n));
  const int r = block_lu<T>(mats + (size_t)s * n * n, n, perm + (size_t)s * n, smem, si,
                            scr + (size_t)s * 2 * LuCfg<T>::NB * n, lperm, use_tc ? &tc : nullptr);
  if (threadIdx.x == 0) info[s] = r;
  if (use_tc) tc_teardown(&tc);
}

// Batched LU with a grid capped by the scratch it is given: CTA b factors
// matrices b, b + gridDim.x, ... and uses scratch rows [b * 2*NB*n, ...).
template <typename T>
__global__ void __launch_bounds__(NT) k_lu_batch_strided(T* mats, int n, int* perm, int* info, T* scr, int nsys) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int si[LU_SI_INTS];
  __shared__ int lperm[MAX_NEQ];
  __shared__ TcState tc;
  const bool use_tc = LuSmem<T>::tc_ok(n);
  if (use_tc) tc_setup(&tc, tc_cols_for(n));
  T* my_scr = scr + (size_t)blockIdx.x * 2 * LuCfg<T>::NB * n;
  for (int s = blockIdx.x; s < nsys; s += gridDim.x) {
    const int r = block_lu<T>(mats + (size_t)s * n * n, n, perm + (size_t)s * n, smem, si, my_scr, lperm,
                              use_tc ? &tc : nullptr);
    if (threadIdx.x == 0) info[s] = r;
    __syncthreads();
  }
  if (use_tc) tc_teardown(&tc);
}

// Rates for a batch of systems (ucl_rates_batch): one CTA per system.
__global__ void __launch_bounds__(NT) k_rates(DevNet N, const ucl_model_params* params, double* abund,
                                              const double* av, double* phi, double* rates, int nsys) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Shared sh;
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const int n = N.neq;
  double* y = (double*)smem;
  double* aux = y + n;
  for (int i = threadIdx.x; i < n; i += NT) y[i] = abund[(size_t)s * n + i];
  if (threadIdx.x == 0) {
    sh.P = params[s];
    SysPhys& S = sh.S;
    S.T = sh.P.initialTemp;
    S.Td = S.T;
    S.av = av[s];
    S.phi = phi[s];
    S.h2crp = 0.0;  // the first interval's h2CRPRate
    S.cs = (sh.P.rout - sh.P.rin) * cK.PC / (double)(float)sh.P.points;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    SysPhys& S = sh.S;
    S.dens = y[n - 1];
    S.h2col = 0.5 * y[N.nh2] * S.dens * S.cs;
    S.cocol = 0.5 * y[N.nco] * S.dens * S.cs;
    S.ccol = 0.5 * y[N.nc] * S.dens * S.cs;
    double sb = 0.0, ss = 0.0;
    for (int i = 0; i < N.n_bulk; i++) sb = i == 0 ? y[N.bulk_list[i]] : sb + y[N.bulk_list[i]];
    for (int i = 0; i < N.n_surface; i++) ss = i == 0 ? y[N.surface_list[i]] : ss + y[N.surface_list[i]];
    if (N.n_bulk > 0) y[N.nbulk] = sb;
    if (N.n_surface > 0) y[N.nsurf] = ss;
    S.sm = fmax(1e-30, ss);
    S.sb = fmax(1e-30, sb);
    if (N.n_refr > 0) {
      double r = 0.0;
      for (int i = 0; i < N.n_refr; i++) r += y[N.refr_list[i]];
      S.sb = S.sb - r;
    }
    const double q = cK.NUM_SITES_PER_GRAIN / (cK.GAS_DUST_DENSITY_RATIO * S.sb);
    S.blr = q < 1.0 ? q : 1.0;
    photo_setup(S, sh.P.radfield);
  }
  __syncthreads();
  dev_rates(N, sh.P, sh.S, y, rates + (size_t)s * N.nreac, aux);
  for (int i = threadIdx.x; i < n; i += NT) abund[(size_t)s * n + i] = y[i];
  if (threadIdx.x == 0) phi[s] = sh.S.phi;
}

// RHS (ucl_rhs_batch) or RHS + analytic Jacobian (ucl_jac_batch), one CTA per system.
__global__ void __launch_bounds__(NT) k_rhs_jac(DevNet N, const ucl_model_params* params, const double* yin,
                                                const double* rates, const double* av, double* ydot, double* jac,
                                                double* jpart, int nsys) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Shared sh;
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const int n = N.neq;
  double* y = (double*)smem;
  double* out = y + n;
  double* flux = out + n;
  double* part = flux + N.nreac;
  double* dfa = part + N.nchunk;
  double* dfb = dfa + N.nreac;
  double* vec = dfb + N.nreac;
  for (int i = threadIdx.x; i < n; i += NT) y[i] = yin[(size_t)s * n + i];
  if (threadIdx.x == 0) {
    sh.P = params[s];
    sh.S.av = av[s];
    sh.S.cs = (sh.P.rout - sh.P.rin) * cK.PC / (double)(float)sh.P.points;
    photo_setup(sh.S, sh.P.radfield);
  }
  __syncthreads();
  const double* r = rates + (size_t)s * N.nreac;
  dev_rhs(N, sh.P, sh.S, y, r, out, flux, part, sh.R, jac != nullptr);
  if (ydot)
    for (int i = threadIdx.x; i < n; i += NT) ydot[(size_t)s * n + i] = out[i];
  if (jac)
    dev_jac<false, double>(N, sh.P, sh.S, y, r, nullptr, nullptr, jac + (size_t)s * n * n, flux, dfa, dfb, vec,
                           jpart + (size_t)s * N.njch, sh.R);
}

}  // namespace ucl
