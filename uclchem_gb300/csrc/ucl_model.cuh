// Whole CLOUD models on the device, one per CTA, and the kernels of the C ABI.
//
//   model set-up      physics-core.f90:42-73, cloud.f90:20-31, chemistry.f90:46-141
//   interval loop     wrap.f90:657-690 with cloud.f90:39-51 (updateTargetTime)
//   updateChemistry   chemistry.f90:145-239 (retries, stall detector)
//   integrateODESystem chemistry.f90:241-292 (abstol vector, ISTATE recovery)
//   output rows       io.f90:74-82
#pragma once
#include "ucl_bdf.cuh"

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
    y[N.nbulk] = sb;
    y[N.nsurf] = ss;
    S.sm = fmax(1e-30, ss);
    S.sb = fmax(1e-30, sb);
    const double q = cK.NUM_SITES_PER_GRAIN / (cK.GAS_DUST_DENSITY_RATIO * S.sb);
    S.blr = q < 1.0 ? q : 1.0;
    photo_setup(S, sh.P.radfield);
  }
  __syncthreads();
}

template <typename T>
__device__ void write_row(Ctx<T>& C, int mi, int max_rows, double* phys_out, double* abund_out) {
  Shared& sh = *C.sh;
  const int nspec = C.N->nspec;
  const int row = sh.ms.row;
  double* ab = abund_out + ((size_t)mi * max_rows + row) * nspec;
  for (int i = threadIdx.x; i < nspec; i += NT) ab[i] = C.y[i];
  if (threadIdx.x == 0) {
    double* ph = phys_out + ((size_t)mi * max_rows + row) * UCL_N_PHYS;
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

template <typename T>
__device__ void run_model(Ctx<T>& C, const ucl_model_params* params, const double* start, int mi, int max_rows,
                          double* phys_out, double* abund_out, int* nrows_out, int* flag_out,
                          ucl_model_stats* stats) {
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
    if (P.points != 1 || P.improvedH2CRPDissociation || P.enforceChargeConservation) ms.flag = UCL_PHYSICS_INIT_ERROR;
  }
  __syncthreads();
  const ucl_model_params& P = sh.P;
  // initial abundances (initializeChemistry, chemistry.f90:57-105)
  for (int i = tid; i < n; i += NT) y[i] = 1.0e-30;
  __syncthreads();
  if (start) {
    for (int i = tid; i < n; i += NT) y[i] = start[(size_t)mi * n + i];
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
  if (ms.flag == 0) write_row(C, mi, max_rows, phys_out, abund_out);
  for (;;) {
    if (tid == 0)
      ms.go = (ms.flag == 0) && ((P.endAtFinalDensity && S.dens < P.finalDens) ||
                                 (!P.endAtFinalDensity && ms.tyears < P.finalTime));
    __syncthreads();
    if (!ms.go) break;
    if (tid == 0) {
      const double told = ms.t;
      ms.tyears = ms.t / cK.SECONDS_PER_YEAR;
      ms.target = target_time(ms.tyears, cK.SECONDS_PER_YEAR);
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
        if (ms.row >= max_rows) ms.flag = UCL_NOT_ENOUGH_TIMEPOINTS_ERROR;
      }
    }
    __syncthreads();
    if (ms.flag < 0) break;
    write_row(C, mi, max_rows, phys_out, abund_out);
  }
  if (tid == 0) {
    nrows_out[mi] = ms.row;
    flag_out[mi] = ms.flag;
    if (stats) {
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
      stats[mi] = st;
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
  L.vec = takec(8 * 1024);
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

template <typename T>
struct SlotArrays {
  double* yh;
  double* rate;
  T* J;
  T* P;
  int* perm;
  T* scr;
  T* dinv;
};

template <typename T>
__device__ __forceinline__ Slot<T> slot_of(const SlotArrays<T>& A, int s, int n, int nreac) {
  Slot<T> W;
  W.yh = nullptr;  // shared memory, set by make_ctx
  W.rate = A.rate + (size_t)s * nreac;
  W.J = A.J + (size_t)s * mat_stride(n);
  W.P = A.P + (size_t)s * mat_stride(n);
  W.perm = A.perm + (size_t)s * n;
  W.scr = A.scr + (size_t)s * 2 * LuCfg<T>::NB * n;
  W.dinv = A.dinv + (size_t)s * dinv_elems(n);
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

// Persistent solver: each CTA pulls model indices from a device counter
// (requests in index order, or through `order` when given).  The launch epoch is the first CTA's start
// time.  With an arrival schedule (seconds after the epoch, ascending), a
// request is not started before its arrival; queue and latency times are
// measured from arrival (from the epoch without a schedule).
template <typename T>
__global__ void __launch_bounds__(NT, 1) k_solve_models(DevNet N, const ucl_model_params* params, const double* start,
                                                     int nmodels, int max_rows, double* phys_out, double* abund_out,
                                                     int* nrows_out, int* flag_out, ucl_model_stats* stats,
                                                     SlotArrays<T> ws, int* counter, unsigned long long* epoch,
                                                     const double* arrival_s, const int* order) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Shared sh;
  __shared__ DevNet sN;
  if (threadIdx.x == 0) sN = N;
  const SmemLayout L = smem_layout<T>(N.neq, N.nreac, N.npart);
  __syncthreads();
  Ctx<T> C = make_ctx<T>(&sN, &sh, smem, L, slot_of(ws, blockIdx.x, N.neq, N.nreac));
  if constexpr (sizeof(T) == 4) tc_setup(&sh.tc);
  __shared__ unsigned long long t_epoch;
  if (threadIdx.x == 0) {
    const unsigned long long now = globaltimer_ns();
    const unsigned long long old = atomicCAS(epoch, 0ull, now);
    t_epoch = old ? old : now;
  }
  for (;;) {
    if (threadIdx.x == 0) {
      const int k = atomicAdd(counter, 1);
      sh.ms.model = (order && k < nmodels) ? order[k] : k;
      const int mi = sh.ms.model;
      sh.ms.ta = t_epoch;
      if (mi < nmodels && arrival_s) {
        const double a = arrival_s[mi];
        const unsigned long long ta = t_epoch + (a > 0.0 ? (unsigned long long)(a * 1e9) : 0ull);
        sh.ms.ta = ta;
        for (unsigned it = 0; it < ADMIT_SLEEP_LIMIT && globaltimer_ns() < ta; ++it) __nanosleep(20000);
      }
    }
    __syncthreads();
    const int mi = sh.ms.model;
    if (mi >= nmodels) break;
    run_model<T>(C, params, start, mi, max_rows, phys_out, abund_out, nrows_out, flag_out, stats);
  }
  if constexpr (sizeof(T) == 4) tc_teardown(&sh.tc);
}

// Batched dense LU (ucl_lu_factor_device): one CTA per matrix, the same
// factorisation the solver applies to its Newton matrices.
template <typename T>
__global__ void __launch_bounds__(NT) k_lu_batch(T* mats, int n, int* perm, int* info, T* scr, int nsys) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int si[LU_SI_INTS];
  __shared__ int lperm[MAX_NEQ];
  __shared__ TcState tc;
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const bool use_tc = LuSmem<T>::tc_ok(n);
  if (use_tc) tc_setup(&tc);
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
  if (use_tc) tc_setup(&tc);
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
    y[N.nbulk] = sb;
    y[N.nsurf] = ss;
    S.sm = fmax(1e-30, ss);
    S.sb = fmax(1e-30, sb);
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
                                                int nsys) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Shared sh;
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const int n = N.neq;
  double* y = (double*)smem;
  double* out = y + n;
  double* flux = out + n;
  double* part = flux + N.nreac;
  double* dfa = part + N.npart;
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
                           part, sh.R);
}

}  // namespace ucl
