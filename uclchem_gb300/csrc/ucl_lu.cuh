// Dense LU with partial pivoting and triangular solves for one system per
// CTA (the Newton matrix P = I - h*gamma*J of the BDF corrector; the
// reference factors it with LINPACK DGEFA/DGESL, dvode.f90:11982-12160).
//
// Storage is row-major (P[i*n + j]) so that row interchanges, panel loads and
// the register-tiled trailing update are all coalesced.  The blocked
// right-looking algorithm:
//   for each panel of NB columns:
//     factor the (n-k0) x NB panel in shared memory (warp pivot search,
//     row swap, scaling, rank-1 updates);
//     swap the same rows in the columns outside the panel;
//     U12 = L11^-1 A12 (one thread per column, registers);
//     A22 -= L21 * U12 (register tiles of TM x TN, operands in shared memory).
// The composite row permutation is kept as perm[] so a solve gathers the
// right-hand side in one parallel pass.
#pragma once
#include "ucl_common.cuh"

namespace ucl {

template <typename T>
struct LuCfg;
template <>
struct LuCfg<float> {
  static constexpr int NB = 32, TM = 8, TN = 8;
};
template <>
struct LuCfg<double> {
  static constexpr int NB = 16, TM = 4, TN = 4;
};

// shared-memory bytes the LU needs for an n x n matrix
template <typename T>
__host__ __device__ constexpr size_t lu_smem_bytes(int n) {
  return sizeof(T) * ((size_t)n * (LuCfg<T>::NB + 1) + (size_t)LuCfg<T>::NB * n) + 64;
}

// Factor A (row-major n x n, global) in place.  perm[i] = original row of
// row i after pivoting.  Returns 0 or (first zero pivot index + 1).
template <typename T>
__device__ int block_lu(T* __restrict__ A, int n, int* __restrict__ perm, char* smem, int* s_i) {
  constexpr int NB = LuCfg<T>::NB, TM = LuCfg<T>::TM, TN = LuCfg<T>::TN;
  constexpr int LDP = NB + 1;
  T* sp = (T*)smem;                  // panel [m x LDP]
  T* su = sp + (size_t)n * LDP;      // U12 [NB x ncols]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int info = 0;
  for (int i = tid; i < n; i += NT) perm[i] = i;
  __syncthreads();
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int nb = min(NB, n - k0);
    const int m = n - k0;
    const int ncols = n - k0 - nb;
    for (int idx = tid; idx < m * nb; idx += NT) {
      const int r = idx / nb, c = idx - r * nb;
      sp[r * LDP + c] = A[(size_t)(k0 + r) * n + k0 + c];
    }
    __syncthreads();
    for (int c = 0; c < nb; ++c) {
      if (warp == 0) {
        T best = (T)-1;
        int bi = c;
        for (int r = c + lane; r < m; r += 32) {
          const T v = fabs(sp[r * LDP + c]);
          if (v > best) { best = v; bi = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const T ov = __shfl_xor_sync(0xffffffffu, best, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) s_i[0] = bi;
      }
      __syncthreads();
      const int p = s_i[0];
      const T pv = sp[p * LDP + c];
      if (pv == (T)0) {
        if (info == 0) info = k0 + c + 1;
        if (tid == 0) s_i[1 + c] = c;
        __syncthreads();
        continue;
      }
      if (p != c) {
        for (int j = tid; j < nb; j += NT) {
          const T t = sp[p * LDP + j];
          sp[p * LDP + j] = sp[c * LDP + j];
          sp[c * LDP + j] = t;
        }
        if (tid == 0) {
          const int t = perm[k0 + p];
          perm[k0 + p] = perm[k0 + c];
          perm[k0 + c] = t;
          s_i[1 + c] = p;  // remember the interchange for the other columns
        }
      } else if (tid == 0) {
        s_i[1 + c] = c;
      }
      __syncthreads();
      const T inv = (T)1 / sp[c * LDP + c];
      for (int r = c + 1 + tid; r < m; r += NT) {
        const T l = sp[r * LDP + c] * inv;
        sp[r * LDP + c] = l;
        for (int j = c + 1; j < nb; ++j) sp[r * LDP + j] -= l * sp[c * LDP + j];
      }
      __syncthreads();
    }
    // panel back to A
    for (int idx = tid; idx < m * nb; idx += NT) {
      const int r = idx / nb, c = idx - r * nb;
      A[(size_t)(k0 + r) * n + k0 + c] = sp[r * LDP + c];
    }
    // the same interchanges in the columns outside the panel (rows are
    // contiguous; each thread applies all nb swaps to its own columns)
    for (int j = tid; j < n - nb; j += NT) {
      const int jj = j < k0 ? j : j + nb;
      for (int c = 0; c < nb; ++c) {
        const int p = s_i[1 + c];
        if (p != c) {
          T* ra = A + (size_t)(k0 + c) * n + jj;
          T* rb = A + (size_t)(k0 + p) * n + jj;
          const T t = *ra;
          *ra = *rb;
          *rb = t;
        }
      }
    }
    __syncthreads();
    if (ncols > 0) {
      // U12 = L11^-1 A12
      for (int jj = tid; jj < ncols; jj += NT) {
        T x[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) {
          if (q < nb) {
            T v = A[(size_t)(k0 + q) * n + k0 + nb + jj];
            for (int p = 0; p < q; ++p) v -= sp[q * LDP + p] * x[p];
            x[q] = v;
          }
        }
#pragma unroll
        for (int q = 0; q < NB; ++q) {
          if (q < nb) {
            A[(size_t)(k0 + q) * n + k0 + nb + jj] = x[q];
            su[q * ncols + jj] = x[q];
          }
        }
      }
      __syncthreads();
      // A22 -= L21 * U12
      const int R = m - nb;
      const int TR = (R + TM - 1) / TM, TC = (ncols + TN - 1) / TN;
      for (int t = tid; t < TR * TC; t += NT) {
        const int ti = t / TC, tj = t - ti * TC;
        const int r0 = ti * TM, j0 = tj * TN;
        T acc[TM][TN];
#pragma unroll
        for (int a = 0; a < TM; ++a)
#pragma unroll
          for (int b = 0; b < TN; ++b) {
            const int r = r0 + a, j = j0 + b;
            acc[a][b] = (r < R && j < ncols) ? A[(size_t)(k0 + nb + r) * n + k0 + nb + j] : (T)0;
          }
        for (int q = 0; q < nb; ++q) {
          T av[TM], bv[TN];
#pragma unroll
          for (int a = 0; a < TM; ++a) av[a] = (r0 + a < R) ? sp[(nb + r0 + a) * LDP + q] : (T)0;
#pragma unroll
          for (int b = 0; b < TN; ++b) bv[b] = (j0 + b < ncols) ? su[q * ncols + j0 + b] : (T)0;
#pragma unroll
          for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; ++b) acc[a][b] -= av[a] * bv[b];
        }
#pragma unroll
        for (int a = 0; a < TM; ++a)
#pragma unroll
          for (int b = 0; b < TN; ++b) {
            const int r = r0 + a, j = j0 + b;
            if (r < R && j < ncols) A[(size_t)(k0 + nb + r) * n + k0 + nb + j] = acc[a][b];
          }
      }
    }
    __syncthreads();
  }
  return info;
}

// Solve (LU) x = b in place, x in shared memory (precision T), perm from
// block_lu.  tmp: shared [n] scratch.
template <typename T>
__device__ void block_lusolve(const T* __restrict__ A, int n, const int* __restrict__ perm, T* x, T* tmp) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n; i += NT) tmp[i] = x[perm[i]];
  __syncthreads();
  // forward: unit lower
  for (int k0 = 0; k0 < n; k0 += 32) {
    const int nb = min(32, n - k0);
    if (warp == 0) {
      T Lr[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) Lr[q] = (lane < nb && q < lane) ? A[(size_t)(k0 + lane) * n + k0 + q] : (T)0;
      T xi = lane < nb ? tmp[k0 + lane] : (T)0;
#pragma unroll
      for (int q = 0; q < 31; ++q) {
        const T xq = __shfl_sync(0xffffffffu, xi, q);
        if (lane > q) xi -= Lr[q] * xq;
      }
      if (lane < nb) tmp[k0 + lane] = xi;
    }
    __syncthreads();
    for (int i = k0 + nb + tid; i < n; i += NT) {
      const T* row = A + (size_t)i * n + k0;
      T s = tmp[i];
      for (int q = 0; q < nb; ++q) s -= row[q] * tmp[k0 + q];
      tmp[i] = s;
    }
    __syncthreads();
  }
  // backward: upper
  const int nblk = (n + 31) / 32;
  for (int bk = nblk - 1; bk >= 0; --bk) {
    const int k0 = bk * 32;
    const int nb = min(32, n - k0);
    if (warp == 0) {
      T Ur[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) Ur[q] = (lane < nb && q >= lane && q < nb) ? A[(size_t)(k0 + lane) * n + k0 + q] : (T)0;
      T xi = lane < nb ? tmp[k0 + lane] : (T)0;
#pragma unroll
      for (int q = 31; q >= 0; --q) {
        if (q < nb) {
          if (lane == q) xi = xi / Ur[q];
          const T xq = __shfl_sync(0xffffffffu, xi, q);
          if (lane < q) xi -= Ur[q] * xq;
        }
      }
      if (lane < nb) tmp[k0 + lane] = xi;
    }
    __syncthreads();
    for (int i = tid; i < k0; i += NT) {
      const T* row = A + (size_t)i * n + k0;
      T s = tmp[i];
      for (int q = 0; q < nb; ++q) s -= row[q] * tmp[k0 + q];
      tmp[i] = s;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += NT) x[i] = tmp[i];
  __syncthreads();
}

}  // namespace ucl
