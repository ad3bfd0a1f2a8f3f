// Shared definitions of the GB300 chemistry solver: device table layout,
// physical constants and block-level helpers.
//
// The device tables are compiled on the host (ucl_capi.cu) from the MakeRates
// network (network.f90 + odes.f90 via uclchem_gb300/network.py) into
//  * per-reaction rate recipes (type code + precomputed constants) that follow
//    the block structure of calculateReactionRates (src/fortran_src/rates.f90:21-343);
//  * the flux form of GETYDOT (odes.f90): one flux per reaction and a
//    signed species-row CSR, split into balanced chunks;
//  * the analytic Jacobian's structural entries.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ucl {

#ifndef UCL_NT
#define UCL_NT 256
#endif
constexpr int NT = UCL_NT;       // threads per CTA of the solver kernels
constexpr int NWARP = NT / 32;
constexpr int MAX_NEQ = 520;     // largest NEQ the kernels are compiled for
constexpr int LMAXP = 7;         // Nordsieck columns held (MAXORD+2)
constexpr int MAX_INV = 32;      // most linear invariants the mixed path projects onto
// doubles of the Jacobian's vector scratch: [0, 256) per-row/ice
// coefficients, [256, 512) their scaled copies, [512, 512 + NEQ) one staged
// matrix row
constexpr int JAC_VEC_DOUBLES = 512 + MAX_NEQ + 8;

// Reaction types (the block of calculateReactionRates that last writes the
// reaction's rate; rates.f90:33-342).
enum RType : uint8_t {
  RT_NONE = 0, RT_CRP, RT_PHOTON, RT_CRPHOT, RT_FREEZE, RT_DESOH2, RT_DESCR, RT_DEUVCR,
  RT_CRS, RT_EXRELAX, RT_EXSOLID, RT_THERM, RT_LH, RT_LHDES, RT_ER, RT_ERDES, RT_H2FORM,
  RT_ZERO, RT_BULKSWAP, RT_SURFSWAP, RT_TWOBODY, RT_IONOPOL1, RT_IONOPOL2, RT_GAR,
  RT_EFREEZE,
};

// Term shapes of the generated RHS (uclchem_gb300/network.py SHAPES).
enum Shape : uint8_t {
  SH_DYY = 0, SH_Y, SH_DY, SH_Y_SM, SH_YY, SH_YY_BLR, SH_Y_BLR, SH_DY_SM_Y, SH_Y_TS_SM, SH_DYY_SM,
};

// 16-byte vector type of T and its width
template <typename T>
struct Vec2;
template <>
struct Vec2<float> { using type = float4; static constexpr int W = 4; };
template <>
struct Vec2<double> { using type = double2; static constexpr int W = 2; };

struct DevNet {
  int nspec, neq, nreac, three_phase;
  int n_surface, n_bulk, n_ice;
  const int* surface_list;
  const int* bulk_list;
  // named species (0-based; absent elements point at the density slot)
  int nh, nh2, nhe, nc, ncx, nco, nelec, nsurf, nbulk, nmgx, nsix, nsx, nclx, no, nn, nmg, np,
      nf, nna, nli, npah, nd, n18o, n15n, n13c;
  // named reactions (-1 where the network has none: a generic network has
  // no self-shielded photo reactions)
  int rx_h2hv, rx_cohv, rx_chv, rx_h2crp;
  // positive ions (species names containing '+'), for enforceChargeConservation
  int n_ion;
  const int* ion_list;
  // refractory ice species subtracted from safeBulk at interval start
  int n_refr;
  const int* refr_list;
  // linear invariants of the ODE system (element counts every reaction
  // conserves), for the mixed path's projection of its Newton corrections:
  // species-major entries inv_sp[inv_sp_ptr[i] ..] = invariant << 8 | count,
  // invariant-major entries inv_el[inv_el_ptr[e] ..] = species << 8 | count
  // (count as int8); n_inv = 0 switches the projection off
  int n_inv;
  const int* inv_sp_ptr;
  const unsigned* inv_sp;
  const int* inv_el_ptr;
  const unsigned* inv_el;
  // ---- rates ----
  const uint8_t* rtype;
  const uint8_t* iceflag;  // PHOTON/CRPHOT: 1 surface, 2 bulk reactant; LHDES/ERDES: 1 bulk reactant
  const int* re1;
  const double* alpha;
  const double* beta;
  const double* gama;
  const double* tmin;
  const double* tmax;
  const uint8_t* extrap;
  const double* mass_re1;  // FREEZE/ER: mass of the reactant
  const double* c0;        // per-type constants (see ucl_capi.cu build_tables)
  const double* c1;
  const double* c2;
  const double* c3;
  const double* c4;
  const int* partner;      // LH <-> LHDES, ER <-> ERDES, EFREEZE -> HFREEZE
  const uint8_t* stick;    // FREEZE: 1 = H2 sticking, 2 = H sticking
  const double* gar;       // GAR parameters, 7 per reaction (row of the GAR block)
  int n_fp;
  const int* fp;           // freeze partners
  const int* fp_re1;
  int desoh2_1, descr_1, deuvcr_1, therm_1;  // first reaction of each block, -1 = absent
  // ---- flux form ----
  const uint8_t* fshape;
  const int* fya;
  const int* fyb;
  int swap_lo, swap_hi;    // reactions whose fluxes sum to totalSwap (bulk swap)
  int n_ts;                // surface-swap (shape 8) reactions
  const int* ts_rx;
  // chunked species-row CSR of signed stoichiometric coefficients
  int nchunk;
  const int* ch_row;
  const int* ch_beg;
  const int* ch_end;
  const int* st_rx;
  const float* st_coef;
  // the same tables packed one 32-bit word per item, so the RHS issues
  // fewer and independent loads:
  //   fpack[r]  = shape << 28 | (yb + 1) << 14 | ya
  //   chpack[c] = row << 20 | len << 16 | beg       (len <= 12)
  //   stpack[e] = (coef & 0xff) << 16 | reaction    (coef as int8)
  //   rowch[i]  = nchunks << 16 | first chunk       (every row 0..neq-1)
  const unsigned* fpack;
  const unsigned* chpack;
  const unsigned* stpack;
  const unsigned* rowch;
  // ---- analytic Jacobian ----
  // structural entries: (row, col) with contributions (reaction<<3 | slot, coef)
  // slot 0: d/dY_a, 1: d/dY_b, 2: d/dD, 3: d/dSURFACE via safeMantle, 4: d/dBULK via blr
  int n_jent;
  const int* je_row;
  const int* je_col;
  const int* je_beg;
  const int* je_end;
  const int* jc_key;
  const float* jc_coef;
  int njch;                // chunks of <= 8 contributions (their partial sums
                           // go to a per-slot global buffer of njch doubles)
  int npart;               // max(nchunk, njch)
  int lu_tc;               // FP32 LU trailing update on the tensor cores (1) or the
                           // CUDA cores (0): chosen per network by the context's
                           // autotuner (ucl_capi.cu tune_lu)
  const unsigned* jent;    // nchunks << 16 | first chunk
  const unsigned* jchunk;  // len << 16 | first contribution
  const unsigned* jcpack;  // (coef & 0xff) << 16 | key
  // surface-swap rank-1: rows with A_i = sum_r S_ir k_r ya_r / sm over shape-8 reactions
  int n_arow;
  const int* ar_row;
  const int* ar_beg;
  const int* ar_end;
  const int* ar_rx;
  const float* ar_coef;
  // photo reactions' species rows (for the d rate / d column-density terms)
  int n_ph;                // species rows of the H2 and CO photo reactions
  const int* ph_row;
  const float* ph_c1;      // stoichiometric coefficient in the H2 photodissociation
  const float* ph_c2;      // stoichiometric coefficient in the CO photodissociation
};

// Physical constants (constants.f90:2-19, surfacereactions.f90:11-52).
// Default-REAL literals of the reference are rounded through float.
struct Consts {
  double K_BOLTZ, REDUCED_PLANCK, AMU, PI, PC, SECONDS_PER_YEAR;
  double GRAIN_RADIUS, THERMAL_VEL, GAS_DUST_DENSITY_RATIO, GRAIN_CROSSSECTION_PER_H,
      GRAIN_SURFACEAREA_PER_H, SURFACE_SITE_DENSITY, VDIFF_PREFACTOR, NUM_SITES_PER_GRAIN,
      CHEMICAL_BARRIER_THICKNESS, MAX_GRAIN_TEMP, MIN_SURFACE_ABUND, MIN_ABUND;
  // spline tables (photoreactions.f90:11-41) and their natural-spline second derivatives
  double lam[30], xlam[30], xlam_y2[30];
  double nco_grid[8], nh2_grid[6];
  double sco[7][6], sco_y2[7][6];
  double sco_m[7][7];       // natural-spline second derivatives over N(CO) as a linear map
  double h2_dw, h2_r, h2_t;  // H2 line shielding constants (photoreactions.f90:46-55, 116-123)
  double xl1000;             // tau(1000 A)/tau(V)
};

// ---------------------------------------------------------------------------
// block helpers (all threads of the CTA must call)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NTH>
__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();  // red may still be read by a previous call
  if (l == 0) red[w] = v;
  __syncthreads();
  // every thread adds the warp sums in the same order (identical results)
  double s = red[0];
#pragma unroll
  for (int i = 1; i < NTH / 32; ++i) s += red[i];
  return s;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

}  // namespace ucl
