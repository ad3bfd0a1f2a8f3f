// Batched variable-order BDF integration, one system per CTA.
//
// The step/order/Jacobian decision logic is that of DVODE_F90 called with
// METHOD_FLAG=22 (src/fortran_src/dvode.f90: DVODE 5654-6766, DVHIN
// 6768-6900, DVINDY_CORE 6901, DVSTEP 7180-7613, DVSET 7616-7789 BDF branch,
// DVJUST 7790-7925 BDF branch, DVNLSD 7926-8179, DVJAC 8182-8400), so the
// device solver takes the same decisions the reference takes; the Jacobian
// is the analytic one (dev_jac) instead of DVODE's finite differences and the
// Newton matrix is factored with block_lu (FP64, or FP32 on the
// error-weight-equilibrated matrix).
//
// Around it, one whole CLOUD model per CTA: the output-interval schedule
// (cloud.f90:39-51), the retry/failure logic of updateChemistry and
// integrateODESystem (chemistry.f90:145-292) and the output rows of
// solveAbundances (wrap.f90:549-697, io.f90:74-82).
//
// Control flow is uniform: scalar decisions are taken by thread 0 and
// published through shared memory behind a barrier; vector work is
// block-strided.
#pragma once
#include "ucl_chem.cuh"
#include "ucl_lu.cuh"

namespace ucl {

struct DvState {
  double h, hscal, hu, hnew, rc, rl1, prl1, tn, eta, etamax, etaq, etaqm1, conp, crate, drc, acnrm;
  double el[14], tq[6], tau[14];
  double del, delp, dsm, told, uround, srur, tolsf;
  double cs;    // 2/(1+rc) when rc != 1 (corrector scaling), formed once per Newton solve
  double rtq2;  // 1/tq[2], formed once per accepted step
  int cs_on;
  int nq, l, lmax, maxord, nqwait, newq, newh, kflag, jstart, jcur, icf, ipup, nslp, nslj;
  int nst, nfe, nje, nlu, nni, ncfn, netf, ncf, m, jok, nls_out, state, istate, ierpj, mxstep;
};

struct ModelState {
  double t, target, orig, tyears, abstol_factor, dens, coldens;
  double ctmax, crad, cmass;  // collapse module: maxTime, parcel radius (pc), mass inside it
  int cmode;                  // 0 cloud, 1-4 collapse modes
  int hmode;                  // 0 off, 1-6 hot-core temperature ramp
  int flag, row, loop, fail_count, retries, model, go;
  long long nst, nfe, nje, nlu, nni, ncfn, netf;
  unsigned long long t0, tp;
  unsigned long long ta;       // arrival time of the request (globaltimer ns)
  unsigned long long tacc[5];  // ns in rates, rhs, jac, lu, solve
};

enum { PH_RATES = 0, PH_RHS, PH_JAC, PH_LU, PH_SOLVE };

struct Shared {
  DvState d;
  ModelState ms;
  SysPhys S;
  RhsScal R;
  ucl_model_params P;
  double red[NWARP + 6];  // block sums; [NWARP+1..NWARP+4] scalars of the step control
  int si[LU_SI_INTS];
  int lperm[MAX_NEQ];
  TcState tc;
  double inv_g[MAX_INV], inv_l[MAX_INV];  // invariant residues and multipliers
};

// per-CTA workspace (global memory)
template <typename T>
struct Slot {
  double* yh;    // [LMAXP * n] Nordsieck array, column j at yh + j*n (shared memory)
  double* rate;  // [nreac]
  T* J;          // [n*n] saved Jacobian (row-major; scaled for T=float)
  T* P;          // [n*n] LU factors
  int* perm;     // [n]
  T* scr;        // [2*NB*n] row-interchange staging
  T* dinv;       // [ceil(n/32) * 2 * 1024] inverses of the diagonal blocks of L and U
  double* jpart; // [njch] partial sums of the Jacobian's entry chunks
  double* ginv;  // [n_inv * n_inv] inverse Gram matrix of the invariants (mixed path)
};

template <typename T>
struct Ctx {
  const DevNet* N;
  Shared* sh;
  int n;
  double *y, *savf, *acor, *ewt, *atol, *tmp, *wJ, *wJi;
  T *xs, *xt;
  double *flux, *part, *dfa, *dfb, *vec, *aux;
  char* lu_smem;
  Slot<T> W;
};

__device__ __forceinline__ double bnorm(const double* v, const double* w, int n, double* red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += NT) {
    const double t = v[i] * w[i];
    s += t * t;
  }
  s = block_sum<NT>(s, red);
  return sqrt(s / n);
}

__device__ __forceinline__ void ph_begin(ModelState& ms) {
  if (threadIdx.x == 0) ms.tp = globaltimer_ns();
}
__device__ __forceinline__ void ph_end(ModelState& ms, int k) {
  if (threadIdx.x == 0) ms.tacc[k] += globaltimer_ns() - ms.tp;
}

// y <- P^-1 y with the current factors
template <typename T>
__device__ void lin_solve(Ctx<T>& C, double* y) {
  const int n = C.n;
  ph_begin(C.sh->ms);
  if constexpr (sizeof(T) == 4)
    block_lusolve<T>(C.W.P, n, C.W.perm, C.W.dinv, y, C.wJ, C.wJi, C.xt, (T*)C.lu_smem);
  else
    block_lusolve<T>(C.W.P, n, C.W.perm, C.W.dinv, y, nullptr, nullptr, C.xt, (T*)C.lu_smem);
  ph_end(C.sh->ms, PH_SOLVE);
}

template <typename T>
__device__ __forceinline__ void rhs(Ctx<T>& C, const double* y, double* out, bool jac = false) {
  ph_begin(C.sh->ms);
  dev_rhs(*C.N, C.sh->P, C.sh->S, y, C.W.rate, out, C.flux, C.part, C.sh->R, jac);
  ph_end(C.sh->ms, PH_RHS);
}

// ---------------------------------------------------------------------------
// Conservative projection of the mixed path's Newton corrections.  Every
// reaction conserves the network's invariants c (element counts), so c.f = 0
// and c.J = 0, hence c.P = c for P = I - h*rl1*J: each exact Newton
// correction leaves c.r, r = rl1*(h*f(y) - zn1) - acor, unchanged, and the
// converged corrector has c.acor = -rl1 c.zn1 (zn1 the predicted first
// Nordsieck column), so the invariants hold to FP64 rounding, as in the
// reference's FP64 solve.  The FP32 factors keep c.(P~^-1 r) = c.r only to
// the FP32 solve's error, amplified by cond(P~), and over ~10^6 steps the
// residue adds up (1e-5 relative drift measured on random mass-action
// networks).  At convergence the mixed path therefore removes it:
//   acor <- acor - Q C^T G^-1 g,  g = C (acor + rl1 zn1),  G = C Q C^T,
// Q = diag(1/ewt^2): the smallest change of acor in DVODE's weighted norm
// that gives the exact corrector's invariant component.  G is formed and
// inverted at each Jacobian evaluation (with the error weights of that
// moment), so a step pays two short reductions.

// G and its inverse (Jacobi-scaled Gauss-Jordan, SPD: no pivoting) into
// W.ginv; an invariant whose scaled pivot vanishes voids the projection
// until the next Jacobian (G^-1 = 0).  All threads call.
template <typename T>
__device__ void inv_prepare(Ctx<T>& C) {
  const DevNet& N = *C.N;
  const int E = N.n_inv, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int E2 = 2 * E;
  double* A = reinterpret_cast<double*>(C.lu_smem);  // [E][2E] scratch: the LU area is idle here
  const int npair = E * (E + 1) / 2;
  for (int p = warp; p < npair; p += NWARP) {
    int e = 0, rem = p;
    while (rem >= E - e) { rem -= E - e; ++e; }
    const int f = e + rem;
    double acc = 0.0;
    for (int k = N.inv_el_ptr[e] + lane; k < N.inv_el_ptr[e + 1]; k += 32) {
      const unsigned w = N.inv_el[k];
      const int sp = (int)(w >> 8), ce = (int)(signed char)(w & 0xFFu);
      int cf = 0;
      for (int q = N.inv_sp_ptr[sp]; q < N.inv_sp_ptr[sp + 1]; ++q) {
        const unsigned v = N.inv_sp[q];
        if ((int)(v >> 8) == f) cf = (int)(signed char)(v & 0xFFu);
      }
      if (cf) {
        const double qs = C.wJi[sp] * C.wJi[sp];
        acc += qs * coef_to_double(ce * cf);
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) {
      A[e * E2 + f] = acc;
      A[f * E2 + e] = acc;
    }
  }
  __syncthreads();
  if (warp == 0) {
    // lane j: column j of the scaled G and column E + j of the identity
    const double gjj = lane < E ? A[lane * E2 + lane] : 1.0;
    const double dj = gjj > 0.0 ? 1.0 / sqrt(gjj) : 0.0;
    bool ok = __all_sync(0xffffffffu, lane >= E || gjj > 0.0);
    for (int i = 0; i < E; ++i) {
      const double di = __shfl_sync(0xffffffffu, dj, i);
      if (lane < E) {
        A[i * E2 + lane] = A[i * E2 + lane] * di * dj;
        A[i * E2 + E + lane] = (i == lane) ? 1.0 : 0.0;
      }
    }
    __syncwarp();
    for (int k = 0; k < E && ok; ++k) {
      const double piv = A[k * E2 + k];
      ok = piv > 1e-10;
      if (!ok) break;
      __syncwarp();
      const double ip = 1.0 / piv;
      if (lane < E) {
        A[k * E2 + lane] *= ip;
        A[k * E2 + E + lane] *= ip;
      }
      __syncwarp();
      for (int i = 0; i < E; ++i) {
        if (i == k) continue;
        const double fct = A[i * E2 + k];
        __syncwarp();
        if (lane < E) {
          A[i * E2 + lane] -= fct * A[k * E2 + lane];
          A[i * E2 + E + lane] -= fct * A[k * E2 + E + lane];
        }
        __syncwarp();
      }
    }
    // G^-1 = D (DGD)^-1 D
    for (int i = 0; i < E; ++i) {
      const double di = __shfl_sync(0xffffffffu, dj, i);
      if (lane < E) C.W.ginv[i * E + lane] = ok ? di * A[i * E2 + E + lane] * dj : 0.0;
    }
  }
  __syncthreads();
}

// acor <- acor - Q C^T G^-1 g and y = yh + acor, g = C (acor + rl1 zn1).
// The exact corrector solution has acor = rl1 (h f(y) - zn1) with zn1 the
// predicted first Nordsieck column, so C acor = -rl1 C zn1 (C f = 0); the
// residue g is the part of the Newton iterate's error that breaks the
// invariants.  (Projecting to C acor = 0 instead would keep any invariant
// part of zn1 out of reach of the corrector, which restores zn1 = h f(y)
// after each step; that part then grows through the predictor.)  All
// threads call.
template <typename T>
__device__ void inv_project(Ctx<T>& C) {
  const DevNet& N = *C.N;
  Shared& sh = *C.sh;
  const int E = N.n_inv, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, n = C.n;
  const double* zn1 = C.W.yh + n;
  const double rl1 = sh.d.rl1;
  for (int e = warp; e < E; e += NWARP) {
    double s = 0.0;
    for (int k = N.inv_el_ptr[e] + lane; k < N.inv_el_ptr[e + 1]; k += 32) {
      const unsigned w = N.inv_el[k];
      const int i = (int)(w >> 8);
      s += coef_to_double((signed char)(w & 0xFFu)) * (C.acor[i] + rl1 * zn1[i]);
    }
    s = warp_sum(s);
    if (lane == 0) sh.inv_g[e] = s;
  }
  __syncthreads();
  if (warp == 0) {
    double l = 0.0;
    if (lane < E)
      for (int f = 0; f < E; ++f) l += C.W.ginv[lane * E + f] * sh.inv_g[f];
    if (lane < E) sh.inv_l[lane] = l;
  }
  __syncthreads();
  const double* yh = C.W.yh;
  for (int i = tid; i < n; i += NT) {
    const int b = N.inv_sp_ptr[i], e1 = N.inv_sp_ptr[i + 1];
    if (b == e1) continue;
    double s = 0.0;
    for (int q = b; q < e1; ++q) {
      const unsigned v = N.inv_sp[q];
      s += coef_to_double((signed char)(v & 0xFFu)) * sh.inv_l[v >> 8];
    }
    const double a = C.acor[i] - C.wJi[i] * C.wJi[i] * s;
    C.acor[i] = a;
    C.y[i] = yh[i] + a;
  }
  __syncthreads();
}

// DVJAC (MITER=2 decision logic, analytic J) + P = I - h*rl1*J + LU
template <typename T>
__device__ int dv_jac(Ctx<T>& C) {
  DvState& d = C.sh->d;
  const int tid = threadIdx.x, n = C.n;
  if (d.jok) {
    if (tid == 0) { d.nslj = d.nst; d.jcur = 1; d.nje++; }
    for (int i = tid; i < n; i += NT) { C.wJ[i] = C.ewt[i]; C.wJi[i] = 1.0 / C.ewt[i]; }
    __syncthreads();
    ph_begin(C.sh->ms);
    dev_jac<(sizeof(T) == 4), T>(*C.N, C.sh->P, C.sh->S, C.y, C.W.rate, C.wJ, C.wJi, C.W.J, C.flux, C.dfa,
                                 C.dfb, C.vec, C.W.jpart, C.sh->R);
    if constexpr (sizeof(T) == 4) {
      if (C.N->n_inv > 0) inv_prepare<T>(C);
    }
    ph_end(C.sh->ms, PH_JAC);
  } else {
    if (tid == 0) d.jcur = 0;
    __syncthreads();
  }
  ph_begin(C.sh->ms);
  const T con = (T)(-(d.h * d.rl1));
  form_newton_matrix<T>(C.W.J, C.W.P, n, con);
  if (tid == 0) d.nlu++;
  __syncthreads();
  // LU with partial pivoting in both precisions.  (An explicit FP32 inverse
  // makes each solve one GEMV but its residual error grows like cond(P)^2;
  // on this problem it multiplied Newton convergence failures, so the
  // factors are kept and applied by triangular solves.)
  const int info = block_lu<T>(C.W.P, n, C.W.perm, C.lu_smem, C.sh->si, C.W.scr, C.sh->lperm,
                               (sizeof(T) == 4 && C.N->lu_tc) ? &C.sh->tc : nullptr);
  lu_diag_inverses<T>(C.W.P, n, C.W.dinv, (T*)C.lu_smem);
  __syncthreads();
  ph_end(C.sh->ms, PH_LU);
  return info != 0;
}

// DVNLSD: modified Newton iteration on the corrector.  Returns 0 / -1.
template <typename T>
__device__ int dv_nlsd(Ctx<T>& C, int nflag) {
  DvState& d = C.sh->d;
  const int tid = threadIdx.x, n = C.n;
  double* yh = C.W.yh;
  if (tid == 0) {
    if (d.jstart == 0) d.nslp = 0;
    if (nflag == 0) d.icf = 0;
    if (nflag == -2) d.ipup = 2;
    if (d.jstart == 0 || d.jstart == -1) d.ipup = 2;
    d.drc = fabs(d.rc - 1.0);
    if (d.drc > 0.3 || d.nst >= d.nslp + 20) d.ipup = 2;
  }
  __syncthreads();
  for (;;) {
    if (tid == 0) {
      d.m = 0;
      d.delp = 0.0;
      d.jok = (d.ipup > 0) &&
              (d.nst == 0 || d.nst > d.nslj + 50 || (d.icf == 1 && d.drc < 0.2) || d.icf == 2);
    }
    __syncthreads();
    for (int i = tid; i < n; i += NT) C.y[i] = yh[i];
    __syncthreads();
    rhs(C, C.y, C.savf, d.jok != 0);
    if (tid == 0) d.nfe++;
    if (d.ipup > 0) {
      const int ierpj = dv_jac<T>(C);
      if (tid == 0) { d.ipup = 0; d.rc = 1.0; d.drc = 0.0; d.crate = 1.0; d.nslp = d.nst; d.ierpj = ierpj; }
      __syncthreads();
      if (d.ierpj) goto fail70;
    }
    if (tid == 0) {
      // scalar FP64 once, not in every thread (FP64 issue is costly on this GPU)
      d.cs_on = fabs(d.rc - 1.0) > 0.0;
      d.cs = d.cs_on ? 2.0 / (1.0 + d.rc) : 1.0;
    }
    for (int i = tid; i < n; i += NT) C.acor[i] = 0.0;
    __syncthreads();
    for (;;) {
      {
        const double rl1h = d.rl1 * d.h, rl1 = d.rl1;
        for (int i = tid; i < n; i += NT) C.y[i] = rl1h * C.savf[i] - (rl1 * yh[n + i] + C.acor[i]);
      }
      __syncthreads();
      lin_solve<T>(C, C.y);
      if (tid == 0) d.nni++;
      double del;
      {
        // scale by 2/(1+rc) when rc != 1, weighted norm of the correction,
        // acor += correction, y = yh0 + acor: one pass, one reduction
        const bool scale = d.cs_on != 0;
        const double cs = d.cs;
        double ss = 0.0;
        for (int i = tid; i < n; i += NT) {
          const double yi = scale ? cs * C.y[i] : C.y[i];
          const double t = yi * C.ewt[i];
          ss += t * t;
          const double a = C.acor[i] + yi;
          C.acor[i] = a;
          C.y[i] = yh[i] + a;
        }
        del = sqrt(block_sum<NT>(ss, C.sh->red) / n);
      }
      if (tid == 0) {
        if (d.m != 0) d.crate = fmax(0.3 * d.crate, del / d.delp);
        const double dcon = del * fmin(1.0, d.crate) / d.tq[4];
        d.del = del;
        if (dcon <= 1.0) d.nls_out = 0;
        else {
          d.m++;
          if (d.m == 3) d.nls_out = 2;
          else if (d.m >= 2 && del > 2.0 * d.delp) d.nls_out = 2;
          else { d.delp = del; d.nls_out = 1; }
        }
      }
      __syncthreads();
      if (d.nls_out == 0) {
        if constexpr (sizeof(T) == 4) {
          if (C.N->n_inv > 0) inv_project<T>(C);
        }
        const double acn = (d.m == 0) ? d.del : bnorm(C.acor, C.ewt, n, C.sh->red);
        if (tid == 0) { d.jcur = 0; d.icf = 0; d.acnrm = acn; }
        __syncthreads();
        return 0;
      }
      if (d.nls_out == 2) break;
      rhs(C, C.y, C.savf);
      if (tid == 0) d.nfe++;
    }
    if (d.jcur == 1) goto fail70;
    if (tid == 0) { d.icf = 1; d.ipup = 2; }
    __syncthreads();
  }
fail70:
  if (tid == 0) { d.icf = 2; d.ipup = 2; }
  __syncthreads();
  return -1;
}

// DVSET, BDF coefficients, by warp 0 (all 32 lanes call).  The divisions,
// which dominate this scalar code (FP64 issue is per warp instruction, and
// slow), run three at a time in parallel lanes: the partial step ratios
// h/hsum_j, then the independent quotients of the error constants, then the
// two that depend on those.  The arithmetic (operands and order) is the
// sequential DVSET's, so the results are bit-identical to it.  Also forms
// rl1 = 1/el[2] and rc <- rc * (rl1/prl1), prl1 = rl1 (DVSTEP after DVSET).
__device__ void dv_set_w(DvState& d) {
  const int lane = threadIdx.x & 31;
  const int nq = d.nq, l = d.l;
  const double flotl = (double)l;
  const double kR[8] = {0.0, 1.0, 1.0 / 2.0, 1.0 / 3.0, 1.0 / 4.0, 1.0 / 5.0, 1.0 / 6.0, 1.0 / 7.0};
  // first division step: lane j (1..nq) forms hsum_j = h + tau[1] + ... + tau[j] and h/hsum_j
  double hs = d.h;
  for (int j = 1; j <= nq; ++j)
    if (j <= lane) hs = hs + d.tau[j];
  const double rxl = d.h / hs;
  double rx[6];
#pragma unroll
  for (int j = 1; j <= 5; ++j) rx[j] = __shfl_sync(0xffffffffu, rxl, j);
  // the el recurrence (every lane, identical)
  double el[7];
  for (int i = 0; i < 7; i++) el[i] = 0.0;
  el[1] = 1.0;
  el[2] = 1.0;
  double alph0 = -1.0, ahatn0 = -1.0, rxi = 1.0, rxis = 1.0;
  if (nq != 1) {
    for (int j = 1; j <= nq - 2; j++) {
      rxi = rx[j];
      const int jp1 = j + 1;
      alph0 = alph0 - kR[jp1];
      for (int ib = 1; ib <= jp1; ib++) {
        const int i = (j + 3) - ib;
        el[i] = el[i] + el[i - 1] * rxi;
      }
    }
    alph0 = alph0 - kR[nq];
    rxis = -el[2] - alph0;
    rxi = rx[nq - 1];
    ahatn0 = -el[2] - rxi;
    for (int ib = 1; ib <= nq; ib++) {
      const int i = (nq + 2) - ib;
      el[i] = el[i] + el[i - 1] * rxis;
    }
  }
  const double t1 = 1.0 - ahatn0 + alph0;
  const double t2 = 1.0 + (double)nq * t1;
  const double t3 = alph0 + kR[nq];
  const double t4 = ahatn0 + rxi;
  const double rxn = rx[nq];  // h / hsum_nq, for the order-raise constant
  const double t5 = alph0 - kR[nq + 1];
  const double t6 = ahatn0 - rxn;
  // second division step: independent quotients
  double num, den;
  switch (lane) {
    case 0: num = alph0 * t2; den = t1; break;           // tq[2]
    case 1: num = el[l] * rxi; den = rxis; break;        // then t2 / this: tq[5]
    case 2: num = rxis; den = el[l]; break;              // cnqm1
    case 3: num = t3; den = 1.0 - t4 + t3; break;        // elp (tq[1])
    case 4: num = t2; den = 1.0 - t6 + t5; break;        // elp (tq[3])
    default: num = 1.0; den = el[2]; break;              // rl1
  }
  const double q2 = num / den;
  const double q_tq2 = __shfl_sync(0xffffffffu, q2, 0), q_b = __shfl_sync(0xffffffffu, q2, 1);
  const double q_cnqm1 = __shfl_sync(0xffffffffu, q2, 2), q_elp1 = __shfl_sync(0xffffffffu, q2, 3);
  const double q_elp2 = __shfl_sync(0xffffffffu, q2, 4), rl1 = __shfl_sync(0xffffffffu, q2, 5);
  // third division step: the quotients of quotients
  if (lane == 0) { num = t2; den = q_b; }
  else if (lane == 1) { num = q_elp1; den = q_cnqm1; }
  else { num = rl1; den = d.prl1; }
  const double q3 = num / den;
  const double q_tq5 = __shfl_sync(0xffffffffu, q3, 0), q_tq1 = __shfl_sync(0xffffffffu, q3, 1);
  const double q_rc = __shfl_sync(0xffffffffu, q3, 2);
  if (lane == 0) {
    for (int i = 1; i <= l; i++) d.el[i] = el[i];
    d.tq[2] = fabs(q_tq2);
    d.tq[5] = fabs(q_tq5);
    if (d.nqwait == 1) {
      d.tq[1] = fabs(q_tq1);
      d.tq[3] = fabs(q_elp2 * rxn * (flotl + 1.0) * t5);
    }
    d.tq[4] = 0.1 * d.tq[2];
    d.rl1 = rl1;
    d.rc = d.rc * q_rc;
    d.prl1 = rl1;
  }
  __syncwarp();
}

// DVJUST, BDF branch: el by thread 0, then the Nordsieck update by all
template <typename T>
__device__ void dv_just(Ctx<T>& C, int iord) {
  DvState& d = C.sh->d;
  const int tid = threadIdx.x, n = C.n;
  double* yh = C.W.yh;
  if (d.nq == 2 && iord != 1) return;
  const int nq = d.nq, l = d.l, lmax = d.lmax;
  if (tid == 0) {
    double* el = d.el;
    for (int i = 1; i <= lmax; i++) el[i] = 0.0;
    el[3] = 1.0;
    if (iord != 1) {
      double hsum = 0.0;
      for (int j = 1; j <= nq - 2; j++) {
        hsum = hsum + d.tau[j];
        const double xi = hsum / d.hscal;
        for (int ib = 1; ib <= j + 1; ib++) {
          const int i = (j + 4) - ib;
          el[i] = el[i] * xi + el[i - 1];
        }
      }
    } else {
      double alph0 = -1.0, alph1 = 1.0, prod = 1.0, xiold = 1.0, hsum = d.hscal;
      if (nq != 1) {
        for (int j = 1; j <= nq - 1; j++) {
          const int jp1 = j + 1;
          hsum = hsum + d.tau[jp1];
          const double xi = hsum / d.hscal;
          prod = prod * xi;
          alph0 = alph0 - 1.0 / (double)jp1;
          alph1 = alph1 + 1.0 / xi;
          for (int ib = 1; ib <= jp1; ib++) {
            const int i = (j + 4) - ib;
            el[i] = el[i] * xiold + el[i - 1];
          }
          xiold = xi;
        }
      }
      d.del = (-alph0 - alph1) / prod;  // t1
    }
  }
  __syncthreads();
  if (iord != 1) {
    for (int i = tid; i < n; i += NT) {
      const double yl = yh[(size_t)(l - 1) * n + i];
      for (int j = 3; j <= nq; j++) yh[(size_t)(j - 1) * n + i] = yh[(size_t)(j - 1) * n + i] - yl * d.el[j];
    }
  } else {
    const double t1 = d.del;
    for (int i = tid; i < n; i += NT) {
      const double v = t1 * yh[(size_t)(lmax - 1) * n + i];
      yh[(size_t)l * n + i] = v;
      for (int j = 3; j <= nq + 1; j++) yh[(size_t)(j - 1) * n + i] = yh[(size_t)(j - 1) * n + i] + d.el[j] * v;
    }
  }
  __syncthreads();
}

enum { ST_L60 = 1, ST_L70, ST_DONE };

// DVSTEP: one step attempt sequence until success or failure (kflag).
template <typename T>
__device__ void dv_step(Ctx<T>& C) {
  DvState& d = C.sh->d;
  const int tid = threadIdx.x, n = C.n;
  double* yh = C.W.yh;
  const double ADDON = 1.0e-6, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, ETACF = 0.25, ETAMIN = 0.1,
               ETAMX1 = 1.0e4, ETAMX2 = 10.0, ETAMX3 = 10.0, ETAMXF = 0.2, THRESH = 1.5;
  int nflag = 0;
  if (tid == 0) {
    d.kflag = 0;
    d.told = d.tn;
    d.ncf = 0;
    d.jcur = 0;
    if (d.jstart == 0) {
      d.lmax = d.maxord + 1;
      d.nq = 1;
      d.l = 2;
      d.tau[1] = d.h;
      d.prl1 = 1.0;
      d.rc = 0.0;
      d.etamax = ETAMX1;
      d.nqwait = 2;
      d.hscal = d.h;
      d.state = ST_L70;
    } else {
      d.state = (d.newh == 0) ? ST_L70 : ST_L60;
    }
  }
  __syncthreads();
  if (d.state == ST_L60 && d.newq != d.nq) {
    const int up = d.newq > d.nq;
    dv_just<T>(C, up ? 1 : -1);
    if (tid == 0) { d.nq = d.newq; d.l = d.nq + 1; d.nqwait = d.l; }
    __syncthreads();
  }
  for (;;) {
    if (d.state == ST_L60) {
      const double eta = d.eta;
      for (int i = tid; i < n; i += NT) {
        double r = 1.0;
        for (int j = 2; j <= d.l; j++) {
          r = r * eta;
          yh[(size_t)(j - 1) * n + i] = r * yh[(size_t)(j - 1) * n + i];
        }
      }
      __syncthreads();
      if (tid == 0) { d.h = d.hscal * d.eta; d.hscal = d.h; d.rc = d.rc * d.eta; d.state = ST_L70; }
      __syncthreads();
    }
    // L70: predict
    const int nq = d.nq;
    if (tid == 0) d.tn = d.tn + d.h;
    for (int i = tid; i < n; i += NT) {
      for (int jb = 1; jb <= nq; jb++)
        for (int c = nq - jb; c < nq; c++) yh[(size_t)c * n + i] += yh[(size_t)(c + 1) * n + i];
    }
    if ((tid >> 5) == 0) dv_set_w(d);
    __syncthreads();
    nflag = dv_nlsd<T>(C, nflag);
    if (nflag != 0) {
      for (int i = tid; i < n; i += NT) {
        for (int jb = 1; jb <= nq; jb++)
          for (int c = nq - jb; c < nq; c++) yh[(size_t)c * n + i] -= yh[(size_t)(c + 1) * n + i];
      }
      if (tid == 0) {
        d.ncf++;
        d.ncfn++;
        d.etamax = 1.0;
        d.tn = d.told;
        if (d.ncf == 10) { d.kflag = -2; d.state = ST_DONE; }
        else { d.eta = ETACF; d.state = ST_L60; }
      }
      __syncthreads();
      if (d.state == ST_DONE) break;
      nflag = -1;
      continue;
    }
    if (tid == 0) d.dsm = d.acnrm / d.tq[2];
    __syncthreads();
    if (d.dsm <= 1.0) {
      // accepted
      const int l = d.l;
      for (int i = tid; i < n; i += NT) {
        const double a = C.acor[i];
        for (int j = 1; j <= l; j++) yh[(size_t)(j - 1) * n + i] += d.el[j] * a;
      }
      if (tid == 0) {
        d.kflag = 0;
        d.nst++;
        d.hu = d.h;
        for (int ib = 1; ib <= d.nq; ib++) {
          const int i = d.l - ib;
          d.tau[i + 1] = d.tau[i];
        }
        d.tau[1] = d.h;
        d.nqwait--;
        d.state = (!((d.l == d.lmax) || (d.nqwait != 1))) ? 1 : 0;  // save acor for an order increase
        if (d.state) d.conp = d.tq[5];
        d.rtq2 = 1.0 / d.tq[2];
      }
      __syncthreads();
      if (d.state) {
        for (int i = tid; i < n; i += NT) yh[(size_t)(d.lmax - 1) * n + i] = C.acor[i];
      }
      __syncthreads();
      if (!(fabs(d.etamax - 1.0) > 0)) {
        if (tid == 0) {
          if (d.nqwait < 2) d.nqwait = 2;
          d.newq = d.nq; d.newh = 0; d.eta = 1.0; d.hnew = d.h;
        }
        __syncthreads();
      } else {
        // L130: order and step selection.  Scalar FP64 (pow) runs in lanes of
        // warp 0 only: one warp-wide pow for the up-to-three candidates.
        const int l = d.l;
        const bool sel = (d.nqwait == 0);
        const int lane = tid & 31, warp = tid >> 5;
        double ddn = 0.0, dup = 0.0;
        if (sel) {
          if (d.nq != 1) ddn = bnorm(yh + (size_t)(l - 1) * n, C.ewt, n, C.sh->red) / d.tq[1];
          if (l != d.lmax) {
            if (tid == 0) C.sh->red[NWARP + 1] = (d.tq[5] / d.conp) * pow(d.h / d.tau[2], (double)l);
            __syncthreads();
            const double cnquot = C.sh->red[NWARP + 1];
            for (int i = tid; i < n; i += NT) C.savf[i] = C.acor[i] - cnquot * yh[(size_t)(d.lmax - 1) * n + i];
            dup = bnorm(C.savf, C.ewt, n, C.sh->red) / d.tq[3];
          }
        }
        if (warp == 0) {
          // lane 0: eta for the same order (etaq); lanes 1, 2: order q-1, q+1
          const double x = BIAS2 * d.dsm;
          // without an order decision, etaq only matters when it reaches
          // THRESH: (BIAS2*dsm)^(1/l) > 1/THRESH - ADDON means it does not
          // (the margin keeps pow's rounding out of the decision)
          double cthr = 1.0 / THRESH - ADDON, thr = cthr;
          for (int k = 1; k < l; ++k) thr *= cthr;
          const bool need_q = sel || !(x > thr * (1.0 + 1e-9));
          const bool need_m = sel && d.nq != 1, need_p = sel && l != d.lmax;
          const bool need = (lane == 0 && need_q) || (lane == 1 && need_m) || (lane == 2 && need_p);
          const double base = lane == 0 ? x : lane == 1 ? BIAS1 * ddn : BIAS3 * dup;
          const double ex = lane == 0 ? 1.0 / (double)l : lane == 1 ? 1.0 / ((double)l - 1.0) : 1.0 / ((double)l + 1.0);
          double r = 0.0;
          if (__any_sync(0xffffffffu, need)) r = need ? 1.0 / (pow(base, ex) + ADDON) : 0.0;
          if (lane < 3) C.sh->red[NWARP + 2 + lane] = r;
        }
        __syncthreads();
        int which = 0;  // 0: keep q, -1: lower, +1: raise
        const double etaq = C.sh->red[NWARP + 2];
        double etaqm1 = C.sh->red[NWARP + 3], etaqp1 = C.sh->red[NWARP + 4];
        if (sel) {
          if (etaq >= etaqp1) which = (etaq < etaqm1) ? -1 : 0;
          else which = (etaqp1 > etaqm1) ? 1 : -1;
          if (which == 1) {
            for (int i = tid; i < n; i += NT) yh[(size_t)(d.lmax - 1) * n + i] = C.acor[i];
          }
        }
        __syncthreads();
        if (tid == 0) {
          d.etaq = etaq;
          if (sel) { d.nqwait = 2; d.etaqm1 = etaqm1; }
          if (which == 0) { d.eta = d.etaq; d.newq = d.nq; }
          else if (which == -1) { d.eta = d.etaqm1; d.newq = d.nq - 1; }
          else { d.eta = etaqp1; d.newq = d.nq + 1; }
          if (d.eta < THRESH || fabs(d.etamax - 1.0) <= 0.0) {
            d.newq = d.nq; d.newh = 0; d.eta = 1.0; d.hnew = d.h;
          } else {
            if (d.eta > d.etamax) d.eta = d.etamax;
            d.newh = 1;
            d.hnew = d.h * d.eta;
          }
        }
        __syncthreads();
      }
      // L250
      if (tid == 0) {
        d.etamax = (d.nst <= 10) ? ETAMX2 : ETAMX3;
      }
      {
        const double r = d.rtq2;
        for (int i = tid; i < n; i += NT) C.acor[i] = r * C.acor[i];
      }
      __syncthreads();
      break;
    }
    // L100: error test failed
    for (int i = tid; i < n; i += NT) {
      for (int jb = 1; jb <= nq; jb++)
        for (int c = nq - jb; c < nq; c++) yh[(size_t)c * n + i] -= yh[(size_t)(c + 1) * n + i];
    }
    if (tid == 0) {
      d.kflag--;
      d.netf++;
      d.tn = d.told;
      d.etamax = 1.0;
      if (d.kflag > -3) {
        double e = 1.0 / (pow(BIAS2 * d.dsm, 1.0 / (double)d.l) + ADDON);
        if (ETAMIN > e) e = ETAMIN;
        if (d.kflag <= -2 && e > ETAMXF) e = ETAMXF;
        d.eta = e;
        d.state = ST_L60;
      } else if (d.kflag == -15) {
        d.kflag = -1;
        d.state = ST_DONE;
      } else if (d.nq != 1) {
        d.eta = ETAMIN;
        d.state = 100;  // lower the order, then L60
      } else {
        d.eta = ETAMIN;
        d.h = d.h * d.eta;
        d.hscal = d.h;
        d.tau[1] = d.h;
        d.state = 120;  // re-evaluate f and restart at order 1
      }
    }
    __syncthreads();
    nflag = -2;
    if (d.state == ST_DONE) break;
    if (d.state == 100) {
      dv_just<T>(C, -1);
      if (tid == 0) { d.l = d.nq; d.nq = d.nq - 1; d.nqwait = d.l; d.state = ST_L60; }
      __syncthreads();
      continue;
    }
    if (d.state == 120) {
      rhs(C, C.y, C.savf);
      const double h = d.h;
      for (int i = tid; i < n; i += NT) yh[n + i] = h * C.savf[i];
      if (tid == 0) { d.nfe++; d.nqwait = 10; d.state = ST_L70; }
      __syncthreads();
      continue;
    }
  }
  if (tid == 0) d.jstart = 1;
  __syncthreads();
}

// DVODE for ITASK=1, ISTATE=1: integrate y from *t to tout.  Returns ISTATE.
template <typename T>
__device__ int dv_ode(Ctx<T>& C, double tout, double rtol) {
  DvState& d = C.sh->d;
  ModelState& ms = C.sh->ms;
  const int tid = threadIdx.x, n = C.n;
  double* yh = C.W.yh;
  double* y = C.y;
  if (fabs(tout - ms.t) <= 0.0) return 1;
  if (tid == 0) {
    d.uround = 2.220446049250313e-16;
    d.srur = sqrt(d.uround);
    d.tn = ms.t;
    d.jstart = 0;
    d.nst = d.nje = d.nni = d.ncfn = d.netf = d.nlu = d.nslj = 0;
    d.nfe = 0;
    d.hu = 0.0;
    d.maxord = 5;
    d.icf = 0; d.ipup = 0; d.nslp = 0; d.newq = 1; d.newh = 0; d.eta = 1.0; d.crate = 1.0; d.drc = 0.0;
    for (int i = 0; i < 14; i++) { d.el[i] = 0.0; d.tau[i] = 0.0; }
    for (int i = 0; i < 6; i++) d.tq[i] = 0.0;
    d.nq = 1;
    d.h = 1.0;
    d.istate = 0;
  }
  for (int i = tid; i < LMAXP * n; i += NT) yh[i] = 0.0;
  __syncthreads();
  rhs(C, y, C.savf);
  int bad = 0;
  for (int i = tid; i < n; i += NT) {
    yh[i] = y[i];
    yh[n + i] = C.savf[i];
    double e = rtol * fabs(y[i]) + C.atol[i];
    if (e <= 0.0) bad = 1;
    C.ewt[i] = 1.0 / e;
  }
  if (tid == 0) d.nfe = 1;
  bad = __syncthreads_or(bad);
  if (bad) return -3;
  // DVHIN: initial step
  {
    const double t0 = ms.t;
    const double tdist = fabs(tout - t0);
    const double tround = d.uround * fmax(fabs(t0), fabs(tout));
    if (tdist < 2.0 * tround) return -3;
    const double hlb = 100.0 * tround;
    double hub = 0.1 * tdist;
    {
      double lim = hub;  // min over i of delyi/afi where afi*hub > delyi
      for (int i = tid; i < n; i += NT) {
        const double delyi = 0.1 * fabs(yh[i]) + C.atol[i];
        const double afi = fabs(yh[n + i]);
        if (afi * hub > delyi) lim = fmin(lim, delyi / afi);
      }
      // block min
      for (int o = 16; o > 0; o >>= 1) lim = fmin(lim, __shfl_xor_sync(0xffffffffu, lim, o));
      __syncthreads();
      if ((tid & 31) == 0) C.sh->red[tid >> 5] = lim;
      __syncthreads();
      double mn = C.sh->red[0];
      for (int w = 1; w < NWARP; w++) mn = fmin(mn, C.sh->red[w]);
      hub = mn;
      __syncthreads();
    }
    double hg = sqrt(hlb * hub), hnew = hg, h0;
    if (hub < hlb) {
      h0 = hg;
    } else {
      int iter = 0;
      for (;;) {
        const double h = copysign(hg, tout - t0);
        for (int i = tid; i < n; i += NT) y[i] = yh[i] + h * yh[n + i];
        __syncthreads();
        rhs(C, y, C.tmp);
        for (int i = tid; i < n; i += NT) C.tmp[i] = (C.tmp[i] - yh[n + i]) / h;
        const double yddnrm = bnorm(C.tmp, C.ewt, n, C.sh->red);
        if (tid == 0) d.nfe++;
        if (yddnrm * hub * hub > 2.0) hnew = sqrt(2.0 / yddnrm);
        else hnew = sqrt(hg * hub);
        iter++;
        if (iter >= 4) break;
        const double hrat = hnew / hg;
        if (hrat > 0.5 && hrat < 2.0) break;
        if (iter >= 2 && hnew > 2.0 * hg) { hnew = hg; break; }
        hg = hnew;
      }
      h0 = hnew * 0.5;
      if (h0 < hlb) h0 = hlb;
      if (h0 > hub) h0 = hub;
    }
    h0 = copysign(h0, tout - t0);
    for (int i = tid; i < n; i += NT) yh[n + i] = h0 * yh[n + i];
    if (tid == 0) d.h = h0;
    __syncthreads();
  }
  int istate = 0;
  bool first = true;
  for (;;) {
    if (!first) {
      if (d.nst >= d.mxstep) { istate = -1; break; }
      int badw = 0;
      for (int i = tid; i < n; i += NT) {
        const double e = rtol * fabs(yh[i]) + C.atol[i];
        if (e <= 0.0) badw = 1;
        C.ewt[i] = 1.0 / e;
      }
      badw = __syncthreads_or(badw);
      if (badw) { istate = -6; break; }
    }
    {
      const double tolsf = d.uround * bnorm(yh, C.ewt, n, C.sh->red);
      if (tolsf > 1.0) {
        if (d.nst == 0) return -3;
        istate = -2;
        break;
      }
    }
    first = false;
    dv_step<T>(C);
    if (d.kflag == -1) { istate = -4; break; }
    if (d.kflag == -2) { istate = -5; break; }
    if ((d.tn - tout) * d.h < 0.0) continue;
    // interpolate at tout (DVINDY_CORE, K=0)
    const double s = (tout - d.tn) / d.h;
    const int nq = d.nq, l = d.l;
    for (int i = tid; i < n; i += NT) {
      double v = yh[(size_t)(l - 1) * n + i];
      for (int jb = 1; jb <= nq; jb++) {
        const int j = nq - jb;
        v = yh[(size_t)j * n + i] + s * v;
      }
      y[i] = v;
    }
    if (tid == 0) ms.t = tout;
    __syncthreads();
    return 2;
  }
  for (int i = tid; i < n; i += NT) y[i] = yh[i];
  if (tid == 0) ms.t = d.tn;
  __syncthreads();
  return istate;
}

}  // namespace ucl
