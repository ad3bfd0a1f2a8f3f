/*
 * TEST INFRASTRUCTURE — CPU oracle for the uclchem_gb300 GPU path.
 *
 * A plain-C, FP64, single-threaded-per-model restatement of the reference's
 * chemistry hot path, used ONLY by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py, to check and time the GPU path against.
 * Nothing in the product links or calls this file.
 *
 * What it restates (reference paths relative to the UCLCHEM project):
 *   - calculateReactionRates            src/fortran_src/rates.f90:21-378
 *   - surface chemistry helpers         src/fortran_src/surfacereactions.f90:33-297
 *   - self-shielded photo rates         src/fortran_src/photoreactions.f90:46-304
 *     (natural cubic splines written from the mathematics)
 *   - F / GETYDOT (term for term)       src/fortran_src/chemistry.f90:294-352,
 *                                       src/fortran_src/odes.f90:6-5181
 *   - DVODE_F90, METHOD_FLAG=22 only    src/fortran_src/dvode.f90 (DVODE 5654,
 *     DVHIN 6768, DVINDY_CORE 6901, DVSTEP 7180, DVSET 7616, DVJUST 7790,
 *     DVNLSD 7926, DVJAC 8182 MITER=2, DGEFA 11982, DGESL 12091,
 *     DEWSET 8981, DVNORM 9021; constants 1874-1911, 6204-6230)
 *   - updateChemistry/integrateODESystem src/fortran_src/chemistry.f90:145-292
 *   - cloud model + solveAbundances loop src/fortran_src/cloud.f90:20-51,
 *                                       physics-core.f90:42-103,
 *                                       wrap.f90:549-697, io.f90:59-83
 *   - get_odes (conservation KAT path)  src/fortran_src/wrap.f90:516-547
 *
 * Default-REAL (single precision) literals of the Fortran are reproduced
 * with SP(x) = (double)(float)x so that FP64 results track the reference.
 * Build with -ffp-contract=off so results do not depend on FMA contraction.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "uclchem_gb300.h"

#define SP(x) ((double)(float)(x))

/* ---------------------------------------------------------------------- */
/* constants.f90:2-19, surfacereactions.f90:11-52, rates.f90:16-18        */
static const double K_BOLTZ = 1.38065040e-16;
static const double REDUCED_PLANCK = 1.054571628e-27;
static const double AMU = 1.66053892e-24;
#define PI_ SP(3.141592654)
static const double PC = 3.086e18;
static const double SECONDS_PER_YEAR = 3.16e7;

static double GRAIN_RADIUS = 1.0e-5;
static double THERMAL_VEL, GAS_DUST_DENSITY_RATIO, GRAIN_CROSSSECTION_PER_H,
    GRAIN_SURFACEAREA_PER_H, VDIFF_PREFACTOR, NUM_SITES_PER_GRAIN;
static const double SURFACE_SITE_DENSITY = 1.5e15;
static const double CHEMICAL_BARRIER_THICKNESS = 1.40e-8;
static const double DIFFUSION_BIND_RATIO = 0.5;
static const double MAX_GRAIN_TEMP = 150.0, MIN_SURFACE_ABUND = 1.0e-20;
static const double MIN_ABUND = 1.0e-30;

static void init_constants(void) {
  const double GAS_DUST_MASS_RATIO = 100.0, GRAIN_DENSITY = 3.0;
  THERMAL_VEL = sqrt(8.0 * K_BOLTZ / (PI_ * AMU));
  GAS_DUST_DENSITY_RATIO =
      (4.0 * PI_ * (GRAIN_RADIUS * GRAIN_RADIUS * GRAIN_RADIUS) * GRAIN_DENSITY * GAS_DUST_MASS_RATIO) /
      (3.0 * AMU);
  GRAIN_CROSSSECTION_PER_H = 0.5 * (7.908e-22 + 8.473e-22);
  GRAIN_SURFACEAREA_PER_H = 4.0 * GRAIN_CROSSSECTION_PER_H;
  VDIFF_PREFACTOR = 2.0 * K_BOLTZ * SURFACE_SITE_DENSITY / PI_ / PI_ / AMU;
  NUM_SITES_PER_GRAIN = GRAIN_RADIUS * GRAIN_RADIUS * SURFACE_SITE_DENSITY * 4.0 * PI_;
}

/* ---------------------------------------------------------------------- */
/* Network (UCLNET01 blob written by uclchem_gb300/network.py)            */
enum { R_PHOTON, R_CRP, R_CRPHOT, R_FREEZE, R_DESORB, R_THERM, R_DESOH2, R_DESCR,
       R_DEUVCR, R_H2FORM, R_ER, R_ERDES, R_LH, R_LHDES, R_BULKSWAP, R_SURFSWAP,
       R_IONOPOL1, R_IONOPOL2, R_CRS, R_EXSOLID, R_EXRELAX, R_GAR, R_TWOBODY, R_NRANGE };
enum { S_NCX, S_NHX, S_NH2, S_NHE, S_NHEX, S_NN, S_NNX, S_NO, S_NOX, S_NC, S_NSIX, S_NSX,
       S_NH2O, S_NCH3OH, S_NCL, S_NCLX, S_NCO, S_NMG, S_NMGX, S_NGH, S_NGH2, S_NGN, S_NGO,
       S_NGOH, S_NSURFACE, S_NBULK, S_NH, S_ND, S_NF, S_NP, S_NS, S_NLI, S_NNA, S_NSI,
       S_NPAH, S_N15N, S_N13C, S_N18O, S_NELEC, S_NFE, S_NSP };
enum { X_H2FORM_CT, X_H2FORM_ERDES, X_H2FORM_ER, X_H2FORM_LH, X_H2FORM_LHDES, X_HFREEZE,
       X_EFREEZE, X_H2_HV, X_H2_CRP, X_H2FREEZE, X_C_HV, X_CO_HV, X_NRX };

typedef struct orc_net {
  int nspec, neq, nreac, three_phase;
  double* mass;
  int* atom_counts;
  int n_surface, n_bulk, n_ice, n_refr;
  int *surface_list, *bulk_list, *ice_list, *gas_ice_list, *refr_list;
  double *binding_energy, *formation_enthalpy;
  int sp[S_NSP], rx[X_NRX];
  int *re, *pr; /* [nreac*3], [nreac*4] 0-based, -1 none */
  double *alpha, *beta, *gama, *min_temps, *max_temps, *reduced_masses;
  int* extrapolate;
  int n_fp;
  int* freeze_partners;
  int n_gar;
  double* gar_params; /* [n_gar*7] */
  int ranges[R_NRANGE][2];
  int n_terms;
  int* terms; /* [n_terms*6] species, sign, rate, shape, ya, yb */
  int n_swap;
  int* swap_terms;
  int n_tr;
  int *tr_surface, *tr_bulk;
  int n_ions;
  int* ions;
  char* blob;
} orc_net;

typedef struct { const char* name; int kind; int64_t count; const void* data; } rec_t;

static int find_rec(const char* blob, size_t size, const char* name, rec_t* out) {
  size_t off = 8;
  while (off + 44 <= size) {
    char nm[33];
    memcpy(nm, blob + off, 32);
    nm[32] = 0;
    uint32_t kind;
    uint64_t count;
    memcpy(&kind, blob + off + 32, 4);
    memcpy(&count, blob + off + 36, 8);
    size_t bytes = (size_t)count * (kind == 1 ? 4 : 8);
    if (strcmp(nm, name) == 0) {
      out->name = name;
      out->kind = (int)kind;
      out->count = (int64_t)count;
      out->data = blob + off + 44;
      return 0;
    }
    off += 44 + bytes;
  }
  return -1;
}

static void* dup_rec(const char* blob, size_t size, const char* name, int kind, int64_t* count) {
  rec_t r;
  if (find_rec(blob, size, name, &r) || r.kind != kind) return NULL;
  size_t bytes = (size_t)r.count * (kind == 1 ? 4 : 8);
  void* p = malloc(bytes ? bytes : 8);
  memcpy(p, r.data, bytes);
  if (count) *count = r.count;
  return p;
}

orc_net* orc_net_load(const char* path) {
  init_constants();
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  size_t size = (size_t)ftell(f);
  fseek(f, 0, SEEK_SET);
  char* blob = (char*)malloc(size);
  if (fread(blob, 1, size, f) != size) { fclose(f); free(blob); return NULL; }
  fclose(f);
  if (size < 8 || memcmp(blob, "UCLNET01", 8) != 0) { free(blob); return NULL; }
  orc_net* n = (orc_net*)calloc(1, sizeof(orc_net));
  int64_t c;
  int* dims = (int*)dup_rec(blob, size, "dims", 1, &c);
  n->nspec = dims[0]; n->nreac = dims[1]; n->three_phase = dims[2]; n->neq = n->nspec + 1;
  free(dims);
  n->mass = (double*)dup_rec(blob, size, "mass", 2, NULL);
  n->atom_counts = (int*)dup_rec(blob, size, "atom_counts", 1, NULL);
  n->surface_list = (int*)dup_rec(blob, size, "surface_list", 1, &c); n->n_surface = (int)c;
  n->bulk_list = (int*)dup_rec(blob, size, "bulk_list", 1, &c); n->n_bulk = (int)c;
  n->ice_list = (int*)dup_rec(blob, size, "ice_list", 1, &c); n->n_ice = (int)c;
  n->gas_ice_list = (int*)dup_rec(blob, size, "gas_ice_list", 1, NULL);
  n->refr_list = (int*)dup_rec(blob, size, "refractory_list", 1, &c); n->n_refr = (int)c;
  n->binding_energy = (double*)dup_rec(blob, size, "binding_energy", 2, NULL);
  n->formation_enthalpy = (double*)dup_rec(blob, size, "formation_enthalpy", 2, NULL);
  int* sp = (int*)dup_rec(blob, size, "sp", 1, NULL);
  memcpy(n->sp, sp, sizeof(n->sp)); free(sp);
  int* rx = (int*)dup_rec(blob, size, "rx", 1, NULL);
  memcpy(n->rx, rx, sizeof(n->rx)); free(rx);
  n->re = (int*)dup_rec(blob, size, "re", 1, NULL);
  n->pr = (int*)dup_rec(blob, size, "pr", 1, NULL);
  n->alpha = (double*)dup_rec(blob, size, "alpha", 2, NULL);
  n->beta = (double*)dup_rec(blob, size, "beta", 2, NULL);
  n->gama = (double*)dup_rec(blob, size, "gama", 2, NULL);
  n->min_temps = (double*)dup_rec(blob, size, "min_temps", 2, NULL);
  n->max_temps = (double*)dup_rec(blob, size, "max_temps", 2, NULL);
  n->reduced_masses = (double*)dup_rec(blob, size, "reduced_masses", 2, NULL);
  n->extrapolate = (int*)dup_rec(blob, size, "extrapolate", 1, NULL);
  n->freeze_partners = (int*)dup_rec(blob, size, "freeze_partners", 1, &c); n->n_fp = (int)c;
  n->gar_params = (double*)dup_rec(blob, size, "gar_params", 2, &c); n->n_gar = (int)(c / 7);
  int* rg = (int*)dup_rec(blob, size, "ranges", 1, NULL);
  memcpy(n->ranges, rg, sizeof(n->ranges)); free(rg);
  n->terms = (int*)dup_rec(blob, size, "terms", 1, &c); n->n_terms = (int)(c / 6);
  n->swap_terms = (int*)dup_rec(blob, size, "swap_terms", 1, &c); n->n_swap = (int)(c / 2);
  n->tr_surface = (int*)dup_rec(blob, size, "tr_surface", 1, &c); n->n_tr = (int)c;
  n->tr_bulk = (int*)dup_rec(blob, size, "tr_bulk", 1, NULL);
  n->blob = blob;
  return n;
}

/* Ion list for enforceChargeConservation (chemistry.f90:114-121) needs
 * species names; the Python side passes the indices. */
void orc_net_set_ions(orc_net* n, int nions, const int* ions) {
  free(n->ions);
  n->ions = (int*)malloc(sizeof(int) * (nions > 0 ? nions : 1));
  memcpy(n->ions, ions, sizeof(int) * nions);
  n->n_ions = nions;
}

void orc_net_free(orc_net* n) {
  if (!n) return;
  void* ptrs[] = {n->mass, n->atom_counts, n->surface_list, n->bulk_list, n->ice_list,
                  n->gas_ice_list, n->refr_list, n->binding_energy, n->formation_enthalpy,
                  n->re, n->pr, n->alpha, n->beta, n->gama, n->min_temps, n->max_temps,
                  n->reduced_masses, n->extrapolate, n->freeze_partners, n->gar_params,
                  n->terms, n->swap_terms, n->tr_surface, n->tr_bulk, n->ions, n->blob};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
  free(n);
}
int orc_net_nspec(const orc_net* n) { return n->nspec; }
int orc_net_nreac(const orc_net* n) { return n->nreac; }

/* ---------------------------------------------------------------------- */
/* Natural cubic spline (second derivatives by the tridiagonal recurrence of
 * a spline with zero end curvature) and its evaluation; used for the
 * extinction curve and the CO self-shielding table
 * (photoreactions.f90:225-271 call these; written here from the maths). */
static void spline_natural(const double* x, const double* y, int n, double* y2) {
  double u[128];
  y2[0] = 0.0;
  u[0] = 0.0;
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) -
            sig * u[i - 1]) /
           p;
  }
  double qn = 0.0, un = 0.0;
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; k--) y2[k] = y2[k] * y2[k + 1] + u[k];
}

static double spline_eval(const double* xa, const double* ya, const double* y2a, int n, double x) {
  /* bracket by bisection over 1-based (0, n+1) as a table search */
  int jlo = 0, jhi = n + 1;
  while (jhi - jlo != 1) {
    int jm = (jhi + jlo) / 2;
    if (x > xa[jm - 1]) jlo = jm; else jhi = jm;
  }
  if (jlo == 0) { jlo = 1; jhi = 2; }
  if (jlo == n) { jlo = n - 1; jhi = n; }
  double h = xa[jhi - 1] - xa[jlo - 1];
  double a = (xa[jhi - 1] - x) / h;
  double b = (x - xa[jlo - 1]) / h;
  return a * ya[jlo - 1] + b * ya[jhi - 1] +
         ((a * a * a - a) * y2a[jlo - 1] + (b * b * b - b) * y2a[jhi - 1]) * (h * h) / 6.0;
}

/* photoreactions.f90:11-24: extinction curve tau(lambda)/tau(V) */
static const double LAMBDA_GRID[30] = {910.0, 950.0, 1000.0, 1050.0, 1110.0, 1180.0, 1250.0, 1390.0,
                                       1490.0, 1600.0, 1700.0, 1800.0, 1900.0, 2000.0, 2100.0, 2190.0,
                                       2300.0, 2400.0, 2500.0, 2740.0, 3440.0, 4000.0, 4400.0, 5500.0,
                                       7000.0, 9000.0, 12500.0, 22000.0, 34000.0, 1.0e9};
static const double XLAMBDA_GRID[30] = {5.76, 5.18, 4.65, 4.16, 3.73, 3.40, 3.11, 2.74, 2.63, 2.62,
                                        2.54, 2.50, 2.58, 2.78, 3.01, 3.12, 2.86, 2.58, 2.35, 2.00,
                                        1.58, 1.42, 1.32, 1.00, 0.75, 0.48, 0.28, 0.12, 0.05, 0.00};
/* photoreactions.f90:31-39: log10 CO shielding table (8 N(CO) x 6 N(H2)),
 * listed column by column as the reference writes it */
static const double NCO_GRID[8] = {12.0, 13.0, 14.0, 15.0, 16.0, 17.0, 18.0, 19.0};
static const double NH2_GRID[6] = {18.0, 19.0, 20.0, 21.0, 22.0, 23.0};
static const double SCO_FLAT[48] = {
    0.000e+00, -1.408e-02, -1.099e-01, -4.400e-01, -1.154e+00, -1.888e+00, -2.760e+00, -4.001e+00,
    -8.539e-02, -1.015e-01, -2.104e-01, -5.608e-01, -1.272e+00, -1.973e+00, -2.818e+00, -4.055e+00,
    -1.451e-01, -1.612e-01, -2.708e-01, -6.273e-01, -1.355e+00, -2.057e+00, -2.902e+00, -4.122e+00,
    -4.559e-01, -4.666e-01, -5.432e-01, -8.665e-01, -1.602e+00, -2.303e+00, -3.146e+00, -4.421e+00,
    -1.303e+00, -1.312e+00, -1.367e+00, -1.676e+00, -2.305e+00, -3.034e+00, -3.758e+00, -5.077e+00,
    -3.883e+00, -3.888e+00, -3.936e+00, -4.197e+00, -4.739e+00, -5.165e+00, -5.441e+00, -6.446e+00};
#define DIMCO 7
#define DIMH2 6

static double g_xl_y2[30];
static double g_sco_rows[DIMCO][DIMH2], g_sco_y2[DIMCO][DIMH2];
static pthread_once_t g_tab_once = PTHREAD_ONCE_INIT;
static void init_tables(void) {
  spline_natural(LAMBDA_GRID, XLAMBDA_GRID, 30, g_xl_y2);
  /* The reference passes the (8,6) table to explicit-shape (7,6) dummies
   * (photoreactions.f90:256,268 -> :306,:406), so element (j,k) of the
   * table it splines is element (k-1)*7+(j-1) of the storage sequence. */
  for (int j = 0; j < DIMCO; j++)
    for (int k = 0; k < DIMH2; k++) g_sco_rows[j][k] = SCO_FLAT[k * DIMCO + j];
  for (int j = 0; j < DIMCO; j++) spline_natural(NH2_GRID, g_sco_rows[j], DIMH2, g_sco_y2[j]);
}

static double xlambda(double lam) { /* photoreactions.f90:225-243 */
  double v = lam;
  if (lam < LAMBDA_GRID[0]) v = LAMBDA_GRID[0];
  if (lam > LAMBDA_GRID[29]) v = LAMBDA_GRID[29];
  double r = spline_eval(LAMBDA_GRID, XLAMBDA_GRID, g_xl_y2, 30, v);
  return r < 0.0 ? 0.0 : r;
}

static double scatter(double x1, double av) { /* photoreactions.f90:133-196 */
  static const double c[6] = {1.0, 2.006, -1.438, 7.364e-01, -5.076e-01, -5.920e-02};
  static const double k1[6] = {7.514e-01, 8.490e-01, 1.013, 1.282, 2.005, 5.832};
  double tv = av / 1.086;
  double tl = tv * xlambda(x1);
  double s = 0.0;
  if (tl < 1.0) {
    double expo = k1[0] * tl;
    if (expo < 100.0) s = c[0] * exp(-expo);
  } else {
    for (int i = 1; i < 6; i++) {
      double expo = k1[i] * tl;
      if (expo < 100.0) s = s + c[i] * exp(-expo);
    }
  }
  return s;
}

static double h2_self_shielding(double nh2, double dw, double rw) { /* photoreactions.f90:91-127 */
  const double FPARA = 0.5, FOSC = 1.0e-2;
  double taud = FPARA * nh2 * SP(1.5e-2) * FOSC / dw;
  double sj, sr;
  if (taud == 0.0) sj = 1.0;
  else if (taud < 2.0) sj = exp(-0.6666667 * taud);
  else if (taud < 10.0) sj = 0.638 * pow(taud, -1.25);
  else if (taud < 100.0) sj = 0.505 * pow(taud, -1.15);
  else sj = 0.344 * pow(taud, -1.0667);
  if (rw == 0.0) sr = 0.0;
  else {
    double r = rw / (1.7724539 * dw);
    double t = 3.02 * pow(r * 1.0e+03, -0.064);
    double u = sqrt(taud * r) / t;
    sr = r / (t * sqrt(0.78539816 + u * u));
  }
  return sj + sr;
}

static double h2_photodiss_rate(double nh2, double radfield, double av, double turbvel) {
  const double baseRate = 5.18e-11, xl = 1000.0, radWidth = 8.0e7; /* photoreactions.f90:46-55 */
  double dw = turbvel / (xl * 1.0e-8);
  return baseRate * (radfield / SP(1.7)) * scatter(xl, av) * h2_self_shielding(nh2, dw, radWidth);
}

static double co_self_shielding(double nh2, double nco) { /* photoreactions.f90:251-271 */
  double lognco = log10(nco + 1.0), lognh2 = log10(nh2 + 1.0);
  if (lognco < NCO_GRID[0]) lognco = NCO_GRID[0];
  if (lognh2 < NH2_GRID[0]) lognh2 = NH2_GRID[0];
  if (lognco > NCO_GRID[DIMCO - 1]) lognco = NCO_GRID[DIMCO - 1];
  if (lognh2 > NH2_GRID[DIMH2 - 1]) lognh2 = NH2_GRID[DIMH2 - 1];
  double yy[DIMCO], y2[DIMCO];
  for (int j = 0; j < DIMCO; j++) yy[j] = spline_eval(NH2_GRID, g_sco_rows[j], g_sco_y2[j], DIMH2, lognh2);
  spline_natural(NCO_GRID, yy, DIMCO, y2);
  double v = spline_eval(NCO_GRID, yy, y2, DIMCO, lognco);
  return pow(10.0, v);
}

static double lbar(double u, double w) { /* photoreactions.f90:275-304 */
  double lu = log10(fabs(u) + 1.0), lw = log10(fabs(w) + 1.0);
  double l = (5675.0 - 200.6 * lw) - (571.6 - 24.09 * lw) * lu + (18.22 - 0.7664 * lw) * (lu * lu);
  if (l > 1076.1) l = 1076.1;
  if (l < 913.6) l = 913.6;
  return l;
}

static double co_photodiss_rate(double nh2, double nco, double radfield, double av) {
  double ssf = co_self_shielding(nh2, nco); /* photoreactions.f90:57-72 */
  double lba = lbar(nco, nh2);
  double sca = scatter(lba, av);
  return (2.e-10) * (radfield / SP(1.7)) * ssf * sca;
}

static double c_ionization_rate(double alpha, double gamma, double T, double nc, double nh2, double av,
                                double radfield) { /* photoreactions.f90:74-85 */
  double tauc = gamma * av + 1.1e-17 * nc + (0.9 * pow(T, 0.27) * pow(nh2 / 1.59e21, 0.45));
  return alpha * (radfield / SP(1.7)) * exp(-tauc);
}

/* ---------------------------------------------------------------------- */
/* surfacereactions.f90:63-107 (Cazaux & Tielens H2 formation)            */
static double h2_form_efficiency(double gasT, double dustT) {
  const double S_MU = 0.005, S_ES = 110.0, S_EH2 = 320.0, S_EHP = 450.0, S_EHC = 3.0e4,
               S_NUH2 = 3.0e12, S_NUHC = 1.3e13, S_CS = 8.473e-22;
  const double G_MU = 0.005, G_ES = 260.0, G_EH2 = 520.0, G_EHP = 800.0, G_EHC = 3.0e4,
               G_NUH2 = 3.0e12, G_NUHC = 1.3e13, G_CS = 7.908e-22;
  double tv = 1.45e5 * sqrt(gasT / 1.0e2);
  double g2 = gasT / 1.0e2;
  double stick = 1.0 / (1.0 + 0.04 * sqrt(gasT + dustT) + 0.2 * (gasT / 1.0e2) + 0.08 * (g2 * g2));
  const double HFLUX = 1.0e-10;
  double f1 = S_MU * HFLUX / (2 * S_NUH2 * exp(-S_EH2 / dustT));
  double q = 1.0 + sqrt((S_EHC - S_ES) / (S_EHP - S_ES));
  double f2 = 1.0 * (q * q) / 4.0 * exp(-S_ES / dustT);
  double eps = 1.0 / (1.0 + S_NUHC / (2 * HFLUX) * exp(-1.5 * S_EHC / dustT) * (q * q));
  double sil = 1.0 / (1.0 + f1 + f2) * eps;
  f1 = G_MU * HFLUX / (2 * G_NUH2 * exp(-G_EH2 / dustT));
  q = 1.0 + sqrt((G_EHC - G_ES) / (G_EHP - G_ES));
  f2 = 1.0 * (q * q) / 4.0 * exp(-G_ES / dustT);
  eps = 1.0 / (1.0 + G_NUHC / (2 * HFLUX) * exp(-1.5 * G_EHC / dustT) * (q * q));
  double gra = 1.0 / (1.0 + f1 + f2) * eps;
  return 0.5 * tv * (S_CS * sil + G_CS * gra) * stick;
}

/* ---------------------------------------------------------------------- */
/* Per-model chemistry state (module globals of the reference, per system) */
typedef struct {
  const orc_net* net;
  ucl_model_params p;
  double gasTemp, dustTemp, density, av, coldens, cloudSize;
  double phi;      /* defaultparameters.f90:117, overwritten by rates.f90:322-326 */
  double lastTemp; /* rates.f90:13 */
  double* rate;    /* [nreac], persists between calls (chemistry.f90:32) */
  double* vdiff;   /* [n_ice] chemistry.f90:108-112 */
  double h2ColToCell, coColToCell, cColToCell;
  double safeMantle, safeBulk, blr;
  double surfaceCoverage_in; /* bulkGainFromMantleBuildUp */
  double h2CRPRate; /* physics-core.f90:15; zero before the first physics update */
} chem_t;

/* x**k, integer k >= 0, by the right-to-left binary method (Knuth TAOCP
 * 4.6.3), as compiled Fortran evaluates a real to a variable integer power */
static double ipow_bin(double x, int k) {
  unsigned e = (unsigned)k;
  double r = (e & 1u) ? x : 1.0;
  while (e >>= 1) {
    x = x * x;
    if (e & 1u) r = r * x;
  }
  return r;
}

/* ionizationDependency's H2 dissociation part (physics-core.f90:121-157),
 * coefficients ckLDiss / ckHDiss of physics-core.f90:29-37 */
static double h2_crp_rate(const ucl_model_params* p, double coldens) {
  static const double cL[10] = {1.582911005330e7, -6.465722684896e6, 1.172189025424e6, -1.237950798073e5,
                                8.393404654312e3, -3.788811358130e2, 1.138688455029e1, -2.197136304567e-1,
                                2.469841278950e-3, -1.232393620924e-5};
  static const double cH[10] = {1.217227462831e7, -4.989649250304e6, 9.079152156645e5, -9.624890825395e4,
                                6.551161486120e3, -2.968976216187e2, 8.959037875226e0, -1.735757324445e-1,
                                1.959267277734e-3, -9.816996707980e-6};
  const double* c = p->ionModel == 'H' ? cH : cL;
  double s = 0.0;
  for (int k = 0; k < 10; k++) s = s + c[k] * ipow_bin(log10(coldens), k);
  return pow(10.0, s) * p->zeta;
}

static double sticking(double s0, double tc, double T) { /* rates.f90:370-378 */
  const double beta = 2.5;
  double tr = T / tc;
  return s0 * (1.0 + beta * tr) / pow(1.0 + tr, beta);
}

static int in_list(const int* list, int n, int v) {
  for (int i = 0; i < n; i++)
    if (list[i] == v) return 1;
  return 0;
}

static double diffusion_reaction_rate(const chem_t* c, int j, double dustT) { /* surfacereactions.f90:158-211 */
  const orc_net* n = c->net;
  int i1 = n->re[3 * j], i2 = n->re[3 * j + 1];
  int idx1 = -1, idx2 = -1;
  for (int i = 0; i < n->n_ice; i++) {
    if (n->ice_list[i] == i1) idx1 = i;
    if (n->ice_list[i] == i2) idx2 = i;
  }
  const double* be = n->binding_energy;
  double diffuse = c->vdiff[idx1] * exp(-DIFFUSION_BIND_RATIO * be[idx1] / dustT);
  diffuse = diffuse + (c->vdiff[idx2] * exp(-DIFFUSION_BIND_RATIO * be[idx2] / dustT));
  double desorb = c->vdiff[idx1] * exp(-be[idx1] / dustT);
  desorb = desorb + c->vdiff[idx2] * exp(-be[idx2] / dustT);
  double reac = n->gama[j] / dustT;
  double rm = n->reduced_masses[j];
  if (rm == 0.0) {
    double m1 = n->mass[n->ice_list[idx1]], m2 = n->mass[n->ice_list[idx2]];
    rm = m1 * m2 / (m1 + m2);
  }
  double tunnel = 2.0 * CHEMICAL_BARRIER_THICKNESS / REDUCED_PLANCK * sqrt(2.0 * AMU * rm * K_BOLTZ * n->gama[j]);
  if (reac > tunnel) reac = tunnel;
  double vmax = c->vdiff[idx1] > c->vdiff[idx2] ? c->vdiff[idx1] : c->vdiff[idx2];
  reac = vmax * exp(-reac);
  reac = reac / (reac + desorb + diffuse);
  return n->alpha[j] * reac * diffuse * GAS_DUST_DENSITY_RATIO / NUM_SITES_PER_GRAIN;
}

static double desorption_fraction(const chem_t* c, int j) { /* surfacereactions.f90:218-297 */
  const orc_net* n = c->net;
  int r1 = n->re[3 * j], r2 = n->re[3 * j + 1];
  int ri1 = 0, ri2 = 0, pi[4] = {0, 0, 0, 0}; /* 1-based ice positions, 0 = none */
  for (int i = 0; i < n->n_ice; i++) {
    int ic = n->ice_list[i], gi = n->gas_ice_list[i];
    if (ic == r1) ri1 = i + 1;
    if (gi == r1) ri1 = i + 1;
    if (ic == r2) ri2 = i + 1;
    if (gi == r2) ri2 = i + 1;
    for (int k = 0; k < 4; k++)
      if (n->pr[4 * j + k] >= 0 && ic == n->pr[4 * j + k]) pi[k] = i + 1;
    for (int k = 0; k < 4; k++)
      if (n->pr[4 * j + k] >= 0 && gi == n->pr[4 * j + k]) pi[k] = i + 1;
  }
  double maxBE = 0.0, prodH = 0.0, epsCd = 0.0;
  for (int k = 0; k < 4; k++) {
    if (pi[k] != 0) {
      double b = n->binding_energy[pi[k] - 1];
      if (b > maxBE) maxBE = b;
      prodH = prodH + n->formation_enthalpy[pi[k] - 1];
      epsCd = epsCd + n->mass[pi[k] - 1]; /* indexed by ice position, as the reference does */
    }
  }
  const double ESM = 120.0;
  double e = (epsCd - ESM) / (epsCd + ESM);
  epsCd = e * e;
  double dH = n->formation_enthalpy[ri1 - 1] + n->formation_enthalpy[ri2 - 1] - prodH;
  dH = dH * 4.184e03 / (1.38054e-23 * 6.02214129e23);
  dH = dH + n->gama[j];
  if (dH == 0.0) dH = SP(1e-30);
  int dof = n->atom_counts[pi[0] - 1];
  for (int k = 1; k < 4; k++)
    if (pi[k] != 0 && n->atom_counts[pi[k] - 1] > dof) dof = n->atom_counts[pi[k] - 1];
  dof = 3 * dof;
  double frac = exp((-maxBE * (double)(float)dof) / (epsCd * dH));
  if (dH < 0.0) frac = 0.0;
  frac = frac / 10;
  const int* sp = n->sp;
  if (r1 == sp[S_NGN] && r2 == sp[S_NGN]) frac = 0.5;
  if ((r1 == sp[S_NGO] && r2 == sp[S_NH]) || (r1 == sp[S_NH] && r2 == sp[S_NGO])) frac = 0.3;
  if ((r1 == sp[S_NGOH] && r2 == sp[S_NH]) || (r1 == sp[S_NH] && r2 == sp[S_NGOH])) frac = 0.25;
  return frac;
}

static void freeze_out(const chem_t* c, int i1, int i2, double* out) { /* rates.f90:354-367 */
  const orc_net* n = c->net;
  for (int j = i1; j <= i2; j++) {
    double fr = 1.0 + n->beta[j - 1] * 16.71e-4 / (GRAIN_RADIUS * c->gasTemp);
    if (c->p.freezeFactor == 0.0 || c->dustTemp > MAX_GRAIN_TEMP) fr = 0.0;
    else
      fr = fr * c->p.freezeFactor * n->alpha[j - 1] * THERMAL_VEL * sqrt(c->gasTemp / n->mass[n->re[3 * (j - 1)]]) *
           GRAIN_CROSSSECTION_PER_H;
    out[j - i1] = fr;
  }
}

static int range_on(const orc_net* n, int r, int* i1, int* i2) {
  *i1 = n->ranges[r][0];
  *i2 = n->ranges[r][1];
  return *i1 != *i2; /* the reference skips a type whose range is one reaction */
}

/* Freeze-out shut-off when a desorption route is much faster
 * (rates.f90:106-107, 127-128, 150-151, 223-224).  The mask runs over the
 * freeze partners' extent. */
static void freeze_shutoff(chem_t* c, const double* abund, int i1, int with_density) {
  const orc_net* n = c->net;
  double* rate = c->rate;
  int nfp = n->n_fp;
  int mask[512];
  for (int k = 0; k < nfp; k++) {
    int fp = n->freeze_partners[k];
    double lhs = rate[fp] * abund[n->re[3 * fp]];
    if (with_density) lhs = lhs * c->density;
    mask[k] = lhs < MIN_SURFACE_ABUND * rate[i1 - 1 + k];
  }
  for (int k = 0; k < nfp; k++)
    if (mask[k]) rate[n->freeze_partners[k]] = 0.0;
}

/* calculateReactionRates, rates.f90:21-343 */
static void calc_rates(chem_t* c, const double* abund, double safeMantle, double h2col, double cocol,
                       double ccol) {
  const orc_net* n = c->net;
  const ucl_model_params* p = &c->p;
  double* rate = c->rate;
  const double T = c->gasTemp, Td = c->dustTemp, av = c->av;
  const double ICE = SP(0.3);
  int i1, i2;
  if (range_on(n, R_CRP, &i1, &i2))
    for (int j = i1; j <= i2; j++) rate[j - 1] = n->alpha[j - 1] * p->zeta;
  if (p->improvedH2CRPDissociation) rate[n->rx[X_H2_CRP]] = c->h2CRPRate; /* rates.f90:38-41 */
  if (range_on(n, R_PHOTON, &i1, &i2)) {
    for (int j = i1; j <= i2; j++) rate[j - 1] = n->alpha[j - 1] * exp(-n->gama[j - 1] * av) * p->radfield / SP(1.7);
    for (int j = i1; j <= i2; j++) {
      int r1 = n->re[3 * (j - 1)];
      if (in_list(n->bulk_list, n->n_bulk, r1))
        rate[j - 1] = rate[j - 1] * ICE * pow((double)(1.0f - 0.007f), 1.0 + 0.5 / c->blr);
      else if (in_list(n->surface_list, n->n_surface, r1))
        rate[j - 1] = rate[j - 1] * ICE;
    }
  }
  if (range_on(n, R_CRPHOT, &i1, &i2)) {
    for (int j = i1; j <= i2; j++)
      rate[j - 1] = n->alpha[j - 1] * n->gama[j - 1] * 1.0 / (1.0 - p->omega) * p->zeta * pow(T / 300, n->beta[j - 1]);
    for (int j = i1; j <= i2; j++) {
      int r1 = n->re[3 * (j - 1)];
      if (in_list(n->bulk_list, n->n_bulk, r1))
        rate[j - 1] = rate[j - 1] * ICE * pow((double)(1.0f - 0.007f), 1 + 0.5 / c->blr);
      else if (in_list(n->surface_list, n->n_surface, r1))
        rate[j - 1] = rate[j - 1] * ICE;
    }
  }
  if (range_on(n, R_FREEZE, &i1, &i2)) {
    freeze_out(c, i1, i2, rate + i1 - 1);
    rate[n->rx[X_EFREEZE]] = rate[n->rx[X_HFREEZE]];
    rate[n->rx[X_H2FREEZE]] = sticking(0.87, 87.0, T) * rate[n->rx[X_H2FREEZE]];
    rate[n->rx[X_HFREEZE]] = sticking(1.0, 52.0, T) * rate[n->rx[X_HFREEZE]];
  }
  if (range_on(n, R_DESOH2, &i1, &i2)) {
    if (p->desorb && p->h2desorb && safeMantle > MIN_SURFACE_ABUND) {
      double v = p->epsilon * h2_form_efficiency(T, Td);
      for (int j = i1; j <= i2; j++) rate[j - 1] = (n->gama[j - 1] > p->ebmaxh2) ? 0.0 : v;
    } else
      for (int j = i1; j <= i2; j++) rate[j - 1] = 0.0;
    freeze_shutoff(c, abund, i1, 0);
  }
  if (range_on(n, R_DESCR, &i1, &i2)) {
    if (p->desorb && p->crdesorb && safeMantle > MIN_SURFACE_ABUND) {
      double v = 4.0 * PI_ * p->zeta * 1.64e-4 * (GRAIN_SURFACEAREA_PER_H) * c->phi;
      for (int j = i1; j <= i2; j++) rate[j - 1] = (n->gama[j - 1] > p->ebmaxcr) ? 0.0 : v;
    } else
      for (int j = i1; j <= i2; j++) rate[j - 1] = 0.0;
    freeze_shutoff(c, abund, i1, 1);
  }
  if (range_on(n, R_DEUVCR, &i1, &i2)) {
    if (p->desorb && p->uvdesorb && safeMantle > MIN_SURFACE_ABUND && p->zeta > 0) {
      double v = GRAIN_CROSSSECTION_PER_H * p->uv_yield * 4.875e3 * p->zeta;
      v = v * (1 + (p->radfield / p->uvcreff) * (1.0 / p->zeta) * exp(SP(-1.8) * av));
      for (int j = i1; j <= i2; j++) rate[j - 1] = (n->gama[j - 1] > p->ebmaxuvcr) ? 0.0 : v;
    } else
      for (int j = i1; j <= i2; j++) rate[j - 1] = 0.0;
    freeze_shutoff(c, abund, i1, 1);
  }
  if (range_on(n, R_CRS, &i1, &i2))
    for (int j = i1; j <= i2; j++)
      rate[j - 1] = n->alpha[j - 1] * (n->beta[j - 1] * (n->gama[j - 1] / 100) * (SP(8.6) * p->zeta * SP(1.3)));
  if (range_on(n, R_EXRELAX, &i1, &i2))
    for (int j = i1; j <= i2; j++)
      for (int i = 0; i < n->n_ice; i++)
        if (n->ice_list[i] == n->re[3 * (j - 1)]) rate[j - 1] = c->vdiff[i];
  if (range_on(n, R_EXSOLID, &i1, &i2))
    for (int j = i1; j <= i2; j++) {
      double vA = 0, vB = 0;
      for (int i = 0; i < n->n_ice; i++) {
        if (n->ice_list[i] == n->re[3 * (j - 1)]) vA = c->vdiff[i];
        if (n->ice_list[i] == n->re[3 * (j - 1) + 1]) vB = c->vdiff[i];
      }
      rate[j - 1] = n->alpha[j - 1] * ((vB + vA) / (SURFACE_SITE_DENSITY * 1.8e-8));
    }
  if (range_on(n, R_THERM, &i1, &i2)) {
    if (p->thermdesorb) {
      for (int j = i1; j <= i2; j++)
        for (int i = 0; i < n->n_ice; i++)
          if (n->ice_list[i] == n->re[3 * (j - 1)]) {
            rate[j - 1] = c->vdiff[i] * exp(-n->gama[j - 1] / Td);
            if (!n->three_phase) rate[j - 1] = rate[j - 1] * 2.0 * SURFACE_SITE_DENSITY * GRAIN_SURFACEAREA_PER_H;
          }
      freeze_shutoff(c, abund, i1, 1);
      if (safeMantle < MIN_SURFACE_ABUND)
        for (int j = i1; j <= i2; j++) rate[j - 1] = 0.0;
    } else
      for (int j = i1; j <= i2; j++) rate[j - 1] = 0.0;
  }
  if (range_on(n, R_LH, &i1, &i2)) {
    int d1 = n->ranges[R_LHDES][0], d2 = n->ranges[R_LHDES][1];
    if (Td < MAX_GRAIN_TEMP && safeMantle > MIN_SURFACE_ABUND) {
      for (int j = i1; j <= i2; j++) rate[j - 1] = diffusion_reaction_rate(c, j - 1, Td);
      for (int k = 0; k <= d2 - d1; k++) rate[d1 - 1 + k] = rate[i1 - 1 + k];
      for (int j = d1; j <= d2; j++) {
        rate[j - 1] = desorption_fraction(c, j - 1) * rate[j - 1];
        if (in_list(n->bulk_list, n->n_bulk, n->re[3 * (j - 1)])) rate[j - 1] = 0.0;
      }
      for (int k = 0; k <= i2 - i1; k++) rate[i1 - 1 + k] = rate[i1 - 1 + k] - rate[d1 - 1 + k];
    } else {
      for (int j = i1; j <= i2; j++) rate[j - 1] = 0.0;
      for (int j = d1; j <= d2; j++) rate[j - 1] = 0.0;
    }
  }
  if (range_on(n, R_ER, &i1, &i2)) {
    int d1 = n->ranges[R_ERDES][0], d2 = n->ranges[R_ERDES][1];
    double tmp[4096];
    freeze_out(c, i1, i2, tmp);
    for (int j = i1; j <= i2; j++) rate[j - 1] = tmp[j - i1] * exp(-n->gama[j - 1] / Td);
    for (int k = 0; k <= d2 - d1; k++) rate[d1 - 1 + k] = rate[i1 - 1 + k];
    for (int j = d1; j <= d2; j++) {
      rate[j - 1] = desorption_fraction(c, j - 1) * rate[j - 1];
      if (in_list(n->bulk_list, n->n_bulk, n->re[3 * (j - 1)])) rate[j - 1] = 0.0;
    }
    for (int k = 0; k <= i2 - i1; k++) rate[i1 - 1 + k] = rate[i1 - 1 + k] - rate[d1 - 1 + k];
  }
  /* PARAMETERIZE_H2FORM = .True. (rates.f90:12, 281-289) */
  rate[n->rx[X_H2FORM_CT]] = h2_form_efficiency(Td, Td);
  rate[n->rx[X_H2FORM_ER]] = 0.0;
  rate[n->rx[X_H2FORM_ERDES]] = 0.0;
  /* bulkSurfaceExchangeReactions, surfacereactions.f90:109-150 */
  if (n->three_phase) {
    int b1 = n->ranges[R_BULKSWAP][0], b2 = n->ranges[R_BULKSWAP][1];
    int s1 = n->ranges[R_SURFSWAP][0], s2 = n->ranges[R_SURFSWAP][1];
    int off = (Td > MAX_GRAIN_TEMP) || (safeMantle < MIN_SURFACE_ABUND);
    for (int i = b1; i <= b2; i++) {
      if (off) rate[i - 1] = 0.0;
      else
        for (int j = 0; j < n->n_ice; j++)
          if (n->ice_list[j] == n->re[3 * (i - 1)]) rate[i - 1] = c->vdiff[j] * exp(-n->binding_energy[j] / Td);
    }
    for (int i = s1; i <= s2; i++) rate[i - 1] = off ? 0.0 : 1.0;
  }
  /* two-body, cached on temperature (rates.f90:295-314) */
  i1 = n->ranges[R_TWOBODY][0];
  i2 = n->ranges[R_TWOBODY][1];
  if (c->lastTemp != T)
    for (int j = i1; j <= i2; j++)
      rate[j - 1] = n->alpha[j - 1] * pow(T / 300., n->beta[j - 1]) * exp(-n->gama[j - 1] / T);
  if (range_on(n, R_IONOPOL1, &i1, &i2))
    for (int j = i1; j <= i2; j++)
      rate[j - 1] = n->alpha[j - 1] * n->beta[j - 1] * (0.62 + 0.4767 * n->gama[j - 1] * sqrt(300.0 / T));
  if (range_on(n, R_IONOPOL2, &i1, &i2))
    for (int j = i1; j <= i2; j++) {
      double g = n->gama[j - 1];
      rate[j - 1] = n->alpha[j - 1] * n->beta[j - 1] * (1.0 + 0.0967 * g * sqrt(300.0 / T) + g * g * 300.0 / (SP(10.526) * T));
    }
  c->lastTemp = T;
  /* grain-assisted recombination parameter; overwrites phi (quirk Q1) */
  {
    double ph = p->radfield * exp(-2.5 * av) * sqrt(T) / (abund[n->neq - 1] * abund[n->sp[S_NELEC]]);
    if (ph < 1e2) ph = 1e2;
    if (ph > 1e6) ph = 1e6;
    c->phi = ph;
    if (range_on(n, R_GAR, &i1, &i2))
      for (int j = i1; j <= i2; j++) {
        const double* g = n->gar_params + 7 * (j - i1);
        rate[j - 1] = 0.6 * n->alpha[j - 1] * g[0] /
                      (1. + g[1] * pow(ph, g[2]) * (1. + g[3] * pow(T, g[4]) * pow(ph, -g[5] - g[6] * log(T))));
      }
  }
  for (int j = 0; j < n->nreac; j++) {
    if (!n->extrapolate[j] && T < n->min_temps[j]) rate[j] = 0.0;
  }
  for (int j = 0; j < n->nreac; j++) {
    if (!n->extrapolate[j] && T > n->max_temps[j]) rate[j] = 0.0;
  }
  rate[n->rx[X_H2_HV]] = h2_photodiss_rate(h2col, p->radfield, av, 1.0);
  rate[n->rx[X_CO_HV]] = co_photodiss_rate(h2col, cocol, p->radfield, av);
  rate[n->rx[X_C_HV]] = c_ionization_rate(n->alpha[n->rx[X_C_HV]], n->gama[n->rx[X_C_HV]], T, ccol, h2col, av,
                                          p->radfield);
}

/* ---------------------------------------------------------------------- */
/* F (chemistry.f90:294-352) with GETYDOT evaluated term for term
 * (odes.f90:6-5181).  If scale != NULL it receives sum |term| per row. */
static double densdot(const ucl_model_params* p, double d) { /* physics-core.f90:90-103 */
  if (d < p->finalDens && p->freefall)
    return p->freefallFactor * pow(pow(d, 4.) / p->initialDens, SP(0.33)) *
           pow(8.4e-30 * p->initialDens * (pow(d / p->initialDens, SP(0.33)) - 1.), 0.5);
  return 0.0;
}

static void rhs_eval(chem_t* c, const double* Y, double* ydot, double* scale) {
  const orc_net* n = c->net;
  const int neq = n->neq, nspec = n->nspec;
  double* rate = c->rate;
  const double D = Y[neq - 1];
  const double cs = c->cloudSize / (double)(float)c->p.points;
  for (int i = 0; i < neq; i++) ydot[i] = 0.0;
  double cocol = c->coColToCell + 0.5 * Y[n->sp[S_NCO]] * D * cs;
  double h2col = c->h2ColToCell + 0.5 * Y[n->sp[S_NH2]] * D * cs;
  rate[n->rx[X_H2_HV]] = h2_photodiss_rate(h2col, c->p.radfield, c->av, 1.0);
  rate[n->rx[X_CO_HV]] = co_photodiss_rate(h2col, cocol, c->p.radfield, c->av);
  double safeMantle = Y[n->sp[S_NSURFACE]] > 1e-30 ? Y[n->sp[S_NSURFACE]] : 1e-30;
  double safeBulk = Y[n->sp[S_NBULK]] > 1e-30 ? Y[n->sp[S_NBULK]] : 1e-30;
  double q = NUM_SITES_PER_GRAIN / (GAS_DUST_DENSITY_RATIO * safeBulk);
  double blr = q < 1.0 ? q : 1.0;
  double surfaceCoverage = 0.5 * GAS_DUST_DENSITY_RATIO / NUM_SITES_PER_GRAIN;
  /* GETYDOT */
  double totalSwap = 0.0;
  for (int k = 0; k < n->n_swap; k++) {
    double t = rate[n->swap_terms[2 * k]] * Y[n->swap_terms[2 * k + 1]] * blr;
    totalSwap = k == 0 ? t : totalSwap + t;
  }
  int k = 0;
  while (k < n->n_terms) {
    int sp = n->terms[6 * k];
    double loss = 0.0, prod = 0.0, sabs = 0.0;
    int first_l = 1, first_p = 1;
    while (k < n->n_terms && n->terms[6 * k] == sp) {
      const int* t = n->terms + 6 * k;
      double r = rate[t[2]], v;
      double ya = Y[t[4]], yb = t[5] >= 0 ? Y[t[5]] : 0.0;
      switch (t[3]) {
        case 0: v = r * D * ya * yb; break;
        case 1: v = r * ya; break;
        case 2: v = r * D * ya; break;
        case 3: v = r * ya / safeMantle; break;
        case 4: v = r * ya * yb; break;
        case 5: v = r * ya * yb * blr; break;
        case 6: v = r * ya * blr; break;
        case 7: v = r * D * ya / safeMantle * yb; break;
        case 8: v = r * ya * totalSwap / safeMantle; break;
        default: v = r * D * ya * yb / safeMantle; break;
      }
      if (t[1] < 0) { loss = first_l ? v : loss + v; first_l = 0; }
      else { prod = first_p ? v : prod + v; first_p = 0; }
      sabs += fabs(v);
      k++;
    }
    ydot[sp] = prod - loss;
    if (scale) scale[sp] = sabs;
  }
  const int nsurf = n->sp[S_NSURFACE], nbulk = n->sp[S_NBULK];
  double s = 0.0;
  for (int i = 0; i < n->n_bulk; i++) s = i == 0 ? ydot[n->bulk_list[i]] : s + ydot[n->bulk_list[i]];
  ydot[nbulk] = s;
  s = 0.0;
  for (int i = 0; i < n->n_surface; i++) s = i == 0 ? ydot[n->surface_list[i]] : s + ydot[n->surface_list[i]];
  ydot[nsurf] = s;
  double y335 = ydot[nsurf];
  if (y335 < 0) {
    double sc = safeBulk / safeMantle;
    if (sc > 1.0) sc = 1.0;
    for (int i = 0; i < n->n_tr; i++)
      ydot[n->tr_surface[i]] = ydot[n->tr_surface[i]] - y335 * sc * Y[n->tr_bulk[i]] / safeBulk;
    for (int i = 0; i < n->n_tr; i++)
      ydot[n->tr_bulk[i]] = ydot[n->tr_bulk[i]] + y335 * sc * Y[n->tr_bulk[i]] / safeBulk;
    if (scale)
      for (int i = 0; i < n->n_tr; i++) {
        double t = fabs(y335 * sc * Y[n->tr_bulk[i]] / safeBulk);
        scale[n->tr_surface[i]] += t;
        scale[n->tr_bulk[i]] += t;
      }
  } else {
    double sc = surfaceCoverage;
    for (int i = 0; i < n->n_tr; i++)
      ydot[n->tr_surface[i]] = ydot[n->tr_surface[i]] - y335 * sc * Y[n->tr_surface[i]];
    for (int i = 0; i < n->n_tr; i++)
      ydot[n->tr_bulk[i]] = ydot[n->tr_bulk[i]] + y335 * sc * Y[n->tr_surface[i]];
    if (scale)
      for (int i = 0; i < n->n_tr; i++) {
        double t = fabs(y335 * sc * Y[n->tr_surface[i]]);
        scale[n->tr_surface[i]] += t;
        scale[n->tr_bulk[i]] += t;
      }
  }
  s = 0.0;
  for (int i = 0; i < n->n_bulk; i++) s = i == 0 ? ydot[n->bulk_list[i]] : s + ydot[n->bulk_list[i]];
  ydot[nbulk] = s;
  s = 0.0;
  for (int i = 0; i < n->n_surface; i++) s = i == 0 ? ydot[n->surface_list[i]] : s + ydot[n->surface_list[i]];
  ydot[nsurf] = s;
  if (scale) {
    double sb = 0.0, ss = 0.0;
    for (int i = 0; i < n->n_bulk; i++) sb += scale[n->bulk_list[i]];
    for (int i = 0; i < n->n_surface; i++) ss += scale[n->surface_list[i]];
    scale[nbulk] = sb;
    scale[nsurf] = ss;
    scale[neq - 1] = 0.0;
  }
  if (c->p.enforceChargeConservation) {
    double e = 0.0;
    for (int i = 0; i < n->n_ions; i++) e += ydot[n->ions[i]];
    ydot[n->sp[S_NELEC]] = e;
  }
  (void)nspec;
  ydot[neq - 1] = densdot(&c->p, Y[neq - 1]);
}

/* ---------------------------------------------------------------------- */
/* DVODE_F90 with METHOD_FLAG=22: BDF, internally generated dense Jacobian
 * saved for reuse, LINPACK LU.  State per call (ISTATE=1 every call).    */
typedef struct {
  int n;
  double *yh, *ewt, *savf, *acor, *wm, *wmj, *ftem; /* yh: (maxord+2) columns of n */
  int* ipvt;
  double h, hscal, hu, hnew, rc, rl1, prl1, tn, eta, etamax, etaq, etaqm1, conp, crate, drc, acnrm;
  double uround, srur, ccmxj, hmin, hmxi;
  double el[14], tq[6], tau[14];
  int nq, l, lmax, maxord, nqwait, newq, newh, kflag, jstart, jcur, icf, ipup, nslp, nslj;
  int nst, nfe, nje, nlu, nni, ncfn, netf, msbj, mxstep, kuth;
  const double* atol;
  double rtol;
  chem_t* chem;
  /* optional right-hand side other than UCLCHEM's F (generic mass-action
   * systems); NULL = rhs_eval on chem */
  void (*fn)(void* ctx, const double* y, double* out);
  void* fctx;
} dv_t;

#define YH(i, j) yh[(size_t)((j)-1) * n + (i)] /* i 0-based row, j 1-based column */

static double dvnorm(int n, const double* v, const double* w) { /* dvode.f90:9021-9057 */
  double s = 0.0;
  for (int i = 0; i < n; i++) {
    double t = v[i] * w[i];
    s = s + t * t;
  }
  return sqrt(s / n);
}

static void dv_rhs(dv_t* d, const double* y, double* out) {
  if (d->fn) d->fn(d->fctx, y, out);
  else rhs_eval(d->chem, y, out, NULL);
}

static void dv_f(dv_t* d, const double* y, double* out) {
  dv_rhs(d, y, out);
  d->nfe++;
}

/* DGEFA, dvode.f90:11982-12090 (column-major, LINPACK pivoting) */
static int dgefa(double* a, int n, int* ipvt) {
  int info = 0;
  for (int k = 0; k < n - 1; k++) {
    double* ak = a + (size_t)k * n;
    int l = k;
    double amax = fabs(ak[k]);
    for (int i = k + 1; i < n; i++)
      if (fabs(ak[i]) > amax) { amax = fabs(ak[i]); l = i; }
    ipvt[k] = l;
    if (fabs(ak[l]) <= 0.0) { info = k + 1; continue; }
    if (l != k) { double t = ak[l]; ak[l] = ak[k]; ak[k] = t; }
    double t = -1.0 / ak[k];
    for (int i = k + 1; i < n; i++) ak[i] = t * ak[i];
    for (int j = k + 1; j < n; j++) {
      double* aj = a + (size_t)j * n;
      double tj = aj[l];
      if (l != k) { aj[l] = aj[k]; aj[k] = tj; }
      for (int i = k + 1; i < n; i++) aj[i] = aj[i] + tj * ak[i];
    }
  }
  ipvt[n - 1] = n - 1;
  if (fabs(a[(size_t)(n - 1) * n + n - 1]) <= 0.0) info = n;
  return info;
}

static void dgesl(const double* a, int n, const int* ipvt, double* b) { /* dvode.f90:12091-12160 */
  for (int k = 0; k < n - 1; k++) {
    int l = ipvt[k];
    double t = b[l];
    if (l != k) { b[l] = b[k]; b[k] = t; }
    const double* ak = a + (size_t)k * n;
    for (int i = k + 1; i < n; i++) b[i] = b[i] + t * ak[i];
  }
  for (int k = n - 1; k >= 0; k--) {
    const double* ak = a + (size_t)k * n;
    b[k] = b[k] / ak[k];
    double t = -b[k];
    for (int i = 0; i < k; i++) b[i] = b[i] + t * ak[i];
  }
}

/* DVSET, BDF branch (dvode.f90:7616-7789, METH=2) */
static void dvset(dv_t* d) {
  double flotl = (double)d->l;
  int nq = d->nq;
  double* el = d->el;
  double* tq = d->tq;
  for (int i = 3; i <= d->l; i++) el[i] = 0.0;
  el[1] = 1.0;
  el[2] = 1.0;
  double alph0 = -1.0, ahatn0 = -1.0, hsum = d->h, rxi = 1.0, rxis = 1.0;
  if (nq != 1) {
    for (int j = 1; j <= nq - 2; j++) {
      hsum = hsum + d->tau[j];
      rxi = d->h / hsum;
      int jp1 = j + 1;
      alph0 = alph0 - 1.0 / (double)jp1;
      for (int ib = 1; ib <= jp1; ib++) {
        int i = (j + 3) - ib;
        el[i] = el[i] + el[i - 1] * rxi;
      }
    }
    alph0 = alph0 - 1.0 / (double)nq;
    rxis = -el[2] - alph0;
    hsum = hsum + d->tau[nq - 1];
    rxi = d->h / hsum;
    ahatn0 = -el[2] - rxi;
    for (int ib = 1; ib <= nq; ib++) {
      int i = (nq + 2) - ib;
      el[i] = el[i] + el[i - 1] * rxis;
    }
  }
  double t1 = 1.0 - ahatn0 + alph0;
  double t2 = 1.0 + (double)nq * t1;
  tq[2] = fabs(alph0 * t2 / t1);
  tq[5] = fabs(t2 / (el[d->l] * rxi / rxis));
  if (d->nqwait == 1) {
    double cnqm1 = rxis / el[d->l];
    double t3 = alph0 + 1.0 / (double)nq;
    double t4 = ahatn0 + rxi;
    double elp = t3 / (1.0 - t4 + t3);
    tq[1] = fabs(elp / cnqm1);
    hsum = hsum + d->tau[nq];
    rxi = d->h / hsum;
    double t5 = alph0 - 1.0 / (double)(nq + 1);
    double t6 = ahatn0 - rxi;
    elp = t2 / (1.0 - t6 + t5);
    tq[3] = fabs(elp * rxi * (flotl + 1.0) * t5);
  }
  tq[4] = 0.1 * tq[2]; /* CORTES */
}

/* DVJUST, BDF branch (dvode.f90:7790-7925, METH=2) */
static void dvjust(dv_t* d, int iord) {
  int n = d->n;
  double* yh = d->yh;
  double* el = d->el;
  if (d->nq == 2 && iord != 1) return;
  int nq = d->nq, l = d->l;
  if (iord != 1) {
    for (int i = 1; i <= d->lmax; i++) el[i] = 0.0;
    el[3] = 1.0;
    double hsum = 0.0;
    for (int j = 1; j <= nq - 2; j++) {
      hsum = hsum + d->tau[j];
      double xi = hsum / d->hscal;
      int jp1 = j + 1;
      for (int ib = 1; ib <= jp1; ib++) {
        int i = (j + 4) - ib;
        el[i] = el[i] * xi + el[i - 1];
      }
    }
    for (int j = 3; j <= nq; j++)
      for (int i = 0; i < n; i++) YH(i, j) = YH(i, j) - YH(i, l) * el[j];
    return;
  }
  for (int i = 1; i <= d->lmax; i++) el[i] = 0.0;
  el[3] = 1.0;
  double alph0 = -1.0, alph1 = 1.0, prod = 1.0, xiold = 1.0, hsum = d->hscal;
  if (nq != 1) {
    for (int j = 1; j <= nq - 1; j++) {
      int jp1 = j + 1;
      hsum = hsum + d->tau[jp1];
      double xi = hsum / d->hscal;
      prod = prod * xi;
      alph0 = alph0 - 1.0 / (double)jp1;
      alph1 = alph1 + 1.0 / xi;
      for (int ib = 1; ib <= jp1; ib++) {
        int i = (j + 4) - ib;
        el[i] = el[i] * xiold + el[i - 1];
      }
      xiold = xi;
    }
  }
  double t1 = (-alph0 - alph1) / prod;
  int lp1 = l + 1;
  for (int i = 0; i < n; i++) YH(i, lp1) = t1 * YH(i, d->lmax);
  for (int j = 3; j <= nq + 1; j++)
    for (int i = 0; i < n; i++) YH(i, j) = YH(i, j) + el[j] * YH(i, lp1);
}

/* DVJAC, MITER=2 with saved Jacobian (dvode.f90:8182-8400) */
static int dvjac(dv_t* d, double* y) {
  int n = d->n;
  double hrl1 = d->h * d->rl1;
  int jok = 1;
  if (d->nst == 0 || d->nst > d->nslj + d->msbj) jok = -1;
  if (d->icf == 1 && d->drc < d->ccmxj) jok = -1;
  if (d->icf == 2) jok = -1;
  if (jok == -1) {
    d->nslj = d->nst;
    d->jcur = 1;
    double fac = dvnorm(n, d->savf, d->ewt);
    double r0 = 1000.0 * fabs(d->h) * d->uround * (double)n * fac;
    if (fabs(r0) <= 0.0) r0 = 1.0;
    for (int j = 0; j < n; j++) {
      double yj = y[j];
      double r = d->srur * fabs(yj);
      double r2 = r0 / d->ewt[j];
      if (r2 > r) r = r2;
      y[j] = y[j] + r;
      fac = 1.0 / r;
      dv_rhs(d, y, d->ftem);
      double* col = d->wm + (size_t)j * n;
      for (int i = 0; i < n; i++) col[i] = (d->ftem[i] - d->savf[i]) * fac;
      y[j] = yj;
    }
    d->nfe += n;
    d->nje++;
    memcpy(d->wmj, d->wm, sizeof(double) * (size_t)n * n);
  } else {
    d->jcur = 0;
    memcpy(d->wm, d->wmj, sizeof(double) * (size_t)n * n);
  }
  double con = -hrl1;
  size_t nn = (size_t)n * n;
  for (size_t i = 0; i < nn; i++) d->wm[i] = con * d->wm[i];
  for (int i = 0; i < n; i++) d->wm[(size_t)i * n + i] += 1.0;
  d->nlu++;
  return dgefa(d->wm, n, d->ipvt) != 0;
}

/* DVNLSD (dvode.f90:7926-8179): modified Newton iteration */
static int dvnlsd(dv_t* d, double* y, int nflag) {
  int n = d->n;
  double* yh = d->yh;
  const int MAXCOR = 3, MSBP = 20;
  const double CCMAX = 0.3, CRDOWN = 0.3, RDIV = 2.0;
  if (d->jstart == 0) d->nslp = 0;
  if (nflag == 0) d->icf = 0;
  if (nflag == -2) d->ipup = 2;
  if (d->jstart == 0 || d->jstart == -1) d->ipup = 2;
  d->drc = fabs(d->rc - 1.0);
  if (d->drc > CCMAX || d->nst >= d->nslp + MSBP) d->ipup = 2;
  for (;;) { /* label 10 */
    int m = 0;
    double delp = 0.0, del;
    for (int i = 0; i < n; i++) y[i] = YH(i, 1);
    dv_f(d, y, d->savf);
    if (d->ipup > 0) {
      int ierpj = dvjac(d, y);
      d->ipup = 0;
      d->rc = 1.0;
      d->drc = 0.0;
      d->crate = 1.0;
      d->nslp = d->nst;
      if (ierpj) goto fail70;
    }
    for (int i = 0; i < n; i++) d->acor[i] = 0.0;
    for (;;) { /* label 30/40 */
      for (int i = 0; i < n; i++) y[i] = (d->rl1 * d->h) * d->savf[i] - (d->rl1 * YH(i, 2) + d->acor[i]);
      dgesl(d->wm, n, d->ipvt, y);
      d->nni++;
      if (fabs(d->rc - 1.0) > 0.0) {
        double cs = 2.0 / (1.0 + d->rc);
        for (int i = 0; i < n; i++) y[i] = cs * y[i];
      }
      del = dvnorm(n, y, d->ewt);
      for (int i = 0; i < n; i++) d->acor[i] = d->acor[i] + y[i];
      for (int i = 0; i < n; i++) y[i] = YH(i, 1) + d->acor[i];
      if (m != 0) {
        double cr = CRDOWN * d->crate;
        d->crate = cr > del / delp ? cr : del / delp;
      }
      double dcon = del * (d->crate < 1.0 ? d->crate : 1.0) / d->tq[4];
      if (dcon <= 1.0) {
        d->jcur = 0;
        d->icf = 0;
        d->acnrm = (m == 0) ? del : dvnorm(n, d->acor, d->ewt);
        return 0;
      }
      m++;
      if (m == MAXCOR) break;
      if (m >= 2 && del > RDIV * delp) break;
      delp = del;
      dv_f(d, y, d->savf);
    }
    /* label 60 */
    if (d->jcur == 1) break;
    d->icf = 1;
    d->ipup = 2;
  }
fail70:
  d->icf = 2;
  d->ipup = 2;
  return -1;
}

/* DVSTEP (dvode.f90:7180-7613) */
static void dvstep(dv_t* d, double* y) {
  int n = d->n;
  double* yh = d->yh;
  const double ADDON = 1.0e-6, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, ETACF = 0.25, ETAMIN = 0.1,
               ETAMX1 = 1.0e4, ETAMX2 = 10.0, ETAMX3 = 10.0, ETAMXF = 0.2, ONEPSM = 1.00001, THRESH = 1.5;
  const int KFC = -3, KFH = -15, MXNCF = 10;
  d->kflag = 0;
  double told = d->tn;
  int ncf = 0;
  d->jcur = 0;
  int nflag = 0;
  double dsm = 0.0;
  int nqnyh;
  if (d->jstart > 0) goto L10;
  /* jstart == 0: first call */
  d->lmax = d->maxord + 1;
  d->nq = 1;
  d->l = 2;
  d->tau[1] = d->h;
  d->prl1 = 1.0;
  d->rc = 0.0;
  d->etamax = ETAMX1;
  d->nqwait = 2;
  d->hscal = d->h;
  goto L70;
L10:
  if (d->kuth == 1) {
    double r = d->h / d->hscal;
    if (r < d->eta) d->eta = r;
    d->newh = 1;
  }
  if (d->newh == 0) goto L70;
  if (d->newq == d->nq) goto L60;
  if (d->newq < d->nq) {
    dvjust(d, -1);
    d->nq = d->newq;
    d->l = d->nq + 1;
    d->nqwait = d->l;
    goto L60;
  }
  if (d->newq > d->nq) {
    dvjust(d, 1);
    d->nq = d->newq;
    d->l = d->nq + 1;
    d->nqwait = d->l;
    goto L60;
  }
L60: {
  double r = 1.0;
  for (int j = 2; j <= d->l; j++) {
    r = r * d->eta;
    for (int i = 0; i < n; i++) YH(i, j) = r * YH(i, j);
  }
  d->h = d->hscal * d->eta;
  d->hscal = d->h;
  d->rc = d->rc * d->eta;
}
L70:
  nqnyh = d->nq * n;
  d->tn = d->tn + d->h;
  /* predict: Pascal triangle on the Nordsieck array */
  for (int jb = 1; jb <= d->nq; jb++) {
    int i1 = nqnyh - jb * n;
    for (int i = i1; i < nqnyh; i++) yh[i] = yh[i] + yh[i + n];
  }
  dvset(d);
  d->rl1 = 1.0 / d->el[2];
  d->rc = d->rc * (d->rl1 / d->prl1);
  d->prl1 = d->rl1;
  nflag = dvnlsd(d, y, nflag);
  if (nflag != 0) {
    ncf++;
    d->ncfn++;
    d->etamax = 1.0;
    d->tn = told;
    for (int jb = 1; jb <= d->nq; jb++) {
      int i1 = nqnyh - jb * n;
      for (int i = i1; i < nqnyh; i++) yh[i] = yh[i] - yh[i + n];
    }
    if (fabs(d->h) <= d->hmin * ONEPSM) goto L230;
    if (ncf == MXNCF) goto L230;
    d->eta = ETACF;
    {
      double e2 = d->hmin / fabs(d->h);
      if (e2 > d->eta) d->eta = e2;
    }
    nflag = -1;
    goto L60;
  }
  dsm = d->acnrm / d->tq[2];
  if (dsm > 1.0) goto L100;
  /* step accepted */
  d->kflag = 0;
  d->nst++;
  d->hu = d->h;
  for (int ib = 1; ib <= d->nq; ib++) {
    int i = d->l - ib;
    d->tau[i + 1] = d->tau[i];
  }
  d->tau[1] = d->h;
  for (int j = 1; j <= d->l; j++)
    for (int i = 0; i < n; i++) YH(i, j) = YH(i, j) + d->el[j] * d->acor[i];
  d->nqwait--;
  if (!((d->l == d->lmax) || (d->nqwait != 1))) {
    for (int i = 0; i < n; i++) YH(i, d->lmax) = d->acor[i];
    d->conp = d->tq[5];
  }
  if (fabs(d->etamax - 1.0) > 0) goto L130;
  if (d->nqwait < 2) d->nqwait = 2;
  d->newq = d->nq;
  d->newh = 0;
  d->eta = 1.0;
  d->hnew = d->h;
  goto L250;
L100: /* error test failed */
  d->kflag--;
  d->netf++;
  nflag = -2;
  d->tn = told;
  for (int jb = 1; jb <= d->nq; jb++) {
    int i1 = nqnyh - jb * n;
    for (int i = i1; i < nqnyh; i++) yh[i] = yh[i] - yh[i + n];
  }
  if (fabs(d->h) <= d->hmin * ONEPSM) goto L220;
  d->etamax = 1.0;
  if (d->kflag <= KFC) goto L110;
  {
    double flotl = (double)d->l;
    d->eta = 1.0 / (pow(BIAS2 * dsm, 1.0 / flotl) + ADDON);
    double e2 = d->hmin / fabs(d->h);
    if (e2 > d->eta) d->eta = e2;
    if (ETAMIN > d->eta) d->eta = ETAMIN;
    if (d->kflag <= -2 && d->eta > ETAMXF) d->eta = ETAMXF;
  }
  goto L60;
L110:
  if (d->kflag == KFH) goto L220;
  if (d->nq == 1) goto L120;
  {
    double e2 = d->hmin / fabs(d->h);
    d->eta = ETAMIN > e2 ? ETAMIN : e2;
  }
  dvjust(d, -1);
  d->l = d->nq;
  d->nq = d->nq - 1;
  d->nqwait = d->l;
  goto L60;
L120: {
  double e2 = d->hmin / fabs(d->h);
  d->eta = ETAMIN > e2 ? ETAMIN : e2;
  d->h = d->h * d->eta;
  d->hscal = d->h;
  d->tau[1] = d->h;
  dv_f(d, y, d->savf);
  for (int i = 0; i < n; i++) YH(i, 2) = d->h * d->savf[i];
  d->nqwait = 10;
  goto L70;
}
L130: {
  double flotl = (double)d->l;
  d->etaq = 1.0 / (pow(BIAS2 * dsm, 1.0 / flotl) + ADDON);
  double etaqp1;
  if (d->nqwait != 0) goto L170;
  d->nqwait = 2;
  d->etaqm1 = 0.0;
  if (d->nq != 1) {
    double ddn = dvnorm(n, &YH(0, d->l), d->ewt) / d->tq[1];
    d->etaqm1 = 1.0 / (pow(BIAS1 * ddn, 1.0 / (flotl - 1.0)) + ADDON);
  }
  etaqp1 = 0.0;
  if (d->l != d->lmax) {
    double cnquot = (d->tq[5] / d->conp) * pow(d->h / d->tau[2], (double)d->l);
    for (int i = 0; i < n; i++) d->savf[i] = d->acor[i] - cnquot * YH(i, d->lmax);
    double dup = dvnorm(n, d->savf, d->ewt) / d->tq[3];
    etaqp1 = 1.0 / (pow(BIAS3 * dup, 1.0 / (flotl + 1.0)) + ADDON);
  }
  if (d->etaq >= etaqp1) {
    if (d->etaq < d->etaqm1) goto L180;
    goto L170;
  }
  if (etaqp1 > d->etaqm1) {
    d->eta = etaqp1;
    d->newq = d->nq + 1;
    for (int i = 0; i < n; i++) YH(i, d->lmax) = d->acor[i];
    goto L200;
  }
  goto L180;
}
L170:
  d->eta = d->etaq;
  d->newq = d->nq;
  goto L200;
L180:
  d->eta = d->etaqm1;
  d->newq = d->nq - 1;
L200:
  if (d->eta < THRESH || fabs(d->etamax - 1.0) <= 0.0) goto L210;
  if (d->eta > d->etamax) d->eta = d->etamax;
  {
    double den = fabs(d->h) * d->hmxi * d->eta;
    d->eta = d->eta / (den > 1.0 ? den : 1.0);
  }
  d->newh = 1;
  d->hnew = d->h * d->eta;
  goto L250;
L210:
  d->newq = d->nq;
  d->newh = 0;
  d->eta = 1.0;
  d->hnew = d->h;
  goto L250;
L220:
  d->kflag = -1;
  goto L260;
L230:
  d->kflag = -2;
  goto L260;
L250:
  d->etamax = ETAMX3;
  if (d->nst <= 10) d->etamax = ETAMX2;
  {
    double r = 1.0 / d->tq[2];
    for (int i = 0; i < n; i++) d->acor[i] = r * d->acor[i];
  }
L260:
  d->jstart = 1;
}

/* DVHIN (dvode.f90:6768-6900): initial step size */
static int dvhin(dv_t* d, double t0, const double* y0, const double* ydot, double tout, double* yw, double* temp,
                 double* h0) {
  int n = d->n;
  double tdist = fabs(tout - t0);
  double tround = d->uround * (fabs(t0) > fabs(tout) ? fabs(t0) : fabs(tout));
  if (tdist < 2.0 * tround) return -1;
  double hlb = 100.0 * tround, hub = 0.1 * tdist;
  for (int i = 0; i < n; i++) {
    double delyi = 0.1 * fabs(y0[i]) + d->atol[i];
    double afi = fabs(ydot[i]);
    if (afi * hub > delyi) hub = delyi / afi;
  }
  int iter = 0;
  double hg = sqrt(hlb * hub), hnew;
  if (hub < hlb) {
    *h0 = hg;
    goto L30;
  }
  for (;;) {
    double h = copysign(hg, tout - t0);
    for (int i = 0; i < n; i++) yw[i] = y0[i] + h * ydot[i];
    dv_f(d, yw, temp);
    for (int i = 0; i < n; i++) temp[i] = (temp[i] - ydot[i]) / h;
    double yddnrm = dvnorm(n, temp, d->ewt);
    if (yddnrm * hub * hub > 2.0) hnew = sqrt(2.0 / yddnrm);
    else hnew = sqrt(hg * hub);
    iter++;
    if (iter >= 4) break;
    double hrat = hnew / hg;
    if (hrat > 0.5 && hrat < 2.0) break;
    if (iter >= 2 && hnew > 2.0 * hg) { hnew = hg; break; }
    hg = hnew;
  }
  *h0 = hnew * 0.5;
  if (*h0 < hlb) *h0 = hlb;
  if (*h0 > hub) *h0 = hub;
L30:
  *h0 = copysign(*h0, tout - t0);
  return 0;
}

typedef struct { int64_t nst, nfe, nje, nlu, nni, ncfn, netf; } dv_counts;

/* DVODE driver for ITASK=1, ISTATE=1 (dvode.f90:5654-6766).  Returns ISTATE. */
/* Optional CPU-time cap of the calling thread's models (a bounded CPU
 * baseline): a model whose integration has used more than the cap stops
 * with ORC_CPU_LIMIT.  0 = no cap.                                        */
#define ORC_CPU_LIMIT (-99)
static __thread double g_cpu_limit = 0.0, g_cpu_start = 0.0;
static double thread_cpu_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_THREAD_CPUTIME_ID, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
void orc_set_cpu_limit(double seconds) { g_cpu_limit = seconds > 0.0 ? seconds : 0.0; }

static int dvode(dv_t* d, double* y, double* t, double tout, dv_counts* cnt) {
  int n = d->n;
  double* yh = d->yh;
  int istate;
  if (fabs(tout - *t) <= 0.0) return 1;
  d->uround = DBL_EPSILON;
  d->srur = sqrt(d->uround);
  d->tn = *t;
  d->jstart = 0;
  d->ccmxj = 0.2;
  d->msbj = 50;
  d->nst = d->nje = d->nni = d->ncfn = d->netf = d->nlu = d->nslj = 0;
  d->hu = 0.0;
  d->kuth = 0;
  d->hmin = 0.0;
  d->hmxi = 0.0;
  d->maxord = 5;
  d->nfe = 0;
  d->icf = 0;
  d->ipup = 0;
  d->nslp = 0;
  d->newq = 1;
  d->newh = 0;
  d->eta = 1.0;
  d->crate = 1.0;
  d->drc = 0.0;
  memset(d->el, 0, sizeof(d->el));
  memset(d->tq, 0, sizeof(d->tq));
  memset(d->tau, 0, sizeof(d->tau));
  memset(yh, 0, sizeof(double) * (size_t)n * (d->maxord + 2));
  dv_f(d, y, &YH(0, 2));
  for (int i = 0; i < n; i++) YH(i, 1) = y[i];
  d->nq = 1;
  d->h = 1.0;
  for (int i = 0; i < n; i++) {
    d->ewt[i] = d->rtol * fabs(YH(i, 1)) + d->atol[i];
    if (d->ewt[i] <= 0.0) { istate = -3; goto done_err; }
    d->ewt[i] = 1.0 / d->ewt[i];
  }
  {
    double h0;
    if (dvhin(d, *t, &YH(0, 1), &YH(0, 2), tout, y, d->acor, &h0)) { istate = -3; goto done_err; }
    d->h = h0;
    for (int i = 0; i < n; i++) YH(i, 2) = h0 * YH(i, 2);
  }
  goto L210;
  for (;;) {
    /* label 200 */
    if (d->nst >= d->mxstep) { istate = -1; goto L410; }
    for (int i = 0; i < n; i++) {
      d->ewt[i] = d->rtol * fabs(YH(i, 1)) + d->atol[i];
      if (d->ewt[i] <= 0.0) { istate = -6; goto L410; }
      d->ewt[i] = 1.0 / d->ewt[i];
    }
  L210: {
    double tolsf = d->uround * dvnorm(n, &YH(0, 1), d->ewt);
    if (tolsf > 1.0) {
      if (d->nst == 0) { istate = -3; goto done_err; }
      istate = -2;
      goto L410;
    }
  }
    dvstep(d, y);
    if (g_cpu_limit > 0.0 && (d->nst & 63) == 0 && thread_cpu_s() - g_cpu_start > g_cpu_limit) {
      istate = ORC_CPU_LIMIT;
      goto L410;
    }
    if (d->kflag == -1) { istate = -4; goto L410; }
    if (d->kflag == -2) { istate = -5; goto L410; }
    if ((d->tn - tout) * d->h < 0.0) continue;
    /* DVINDY_CORE(TOUT, 0): interpolate y at tout from the Nordsieck array */
    {
      double s = (tout - d->tn) / d->h;
      for (int i = 0; i < n; i++) y[i] = YH(i, d->l);
      for (int jb = 1; jb <= d->nq; jb++) {
        int j = d->nq - jb;
        for (int i = 0; i < n; i++) y[i] = YH(i, j + 1) + s * y[i];
      }
    }
    *t = tout;
    istate = 2;
    goto done;
  }
L410:
  for (int i = 0; i < n; i++) y[i] = YH(i, 1);
  *t = d->tn;
done:
done_err:
  if (cnt) {
    cnt->nst += d->nst; cnt->nfe += d->nfe; cnt->nje += d->nje; cnt->nlu += d->nlu;
    cnt->nni += d->nni; cnt->ncfn += d->ncfn; cnt->netf += d->netf;
  }
  return istate;
}

/* ---------------------------------------------------------------------- */
/* Model set-up: coreInitializePhysics + cloud initializePhysics +
 * initializeChemistry (physics-core.f90:42-73, cloud.f90:20-31,
 * chemistry.f90:46-141) */
static int chem_init(chem_t* c, const orc_net* n, const ucl_model_params* p, double* abund, int set_abund) {
  memset(c, 0, sizeof(*c));
  c->net = n;
  c->p = *p;
  /* coreInitializePhysics's start-up checks (physics-core.f90:55-64); points
   * > 1 is rejected as the device path rejects it (the reference's
   * multi-parcel column density reads coldens(0), physics-core.f90:80) */
  if (p->points != 1 || (p->ionModel != 'L' && p->ionModel != 'H') ||
      (p->improvedH2CRPDissociation && !p->cosmicRayAttenuation))
    return -1;
  c->cloudSize = (p->rout - p->rin) * PC;
  c->gasTemp = p->initialTemp;
  c->dustTemp = c->gasTemp;
  c->density = p->initialDens;
  c->coldens = (double)(float)(p->points - 1 + 1) * c->cloudSize / (double)(float)p->points * p->initialDens;
  c->av = p->baseAv + c->coldens / 1.6e21;
  if (p->freefall) c->density = SP(1.001) * p->initialDens;
  c->phi = p->phi;
  c->lastTemp = 99.0e99;
  c->rate = (double*)calloc((size_t)n->nreac, sizeof(double));
  c->vdiff = (double*)calloc((size_t)n->n_ice, sizeof(double));
  for (int i = 0; i < n->n_ice; i++) {
    int j = n->ice_list[i];
    c->vdiff[i] = sqrt(VDIFF_PREFACTOR * n->binding_energy[i] / n->mass[j]);
  }
  if (set_abund) {
    const int* s = n->sp;
    int neq = n->neq;
    for (int i = 0; i < neq; i++) abund[i] = MIN_ABUND;
    abund[s[S_NO]] = p->fo;
    abund[s[S_NN]] = p->fn;
    abund[s[S_NMG]] = p->fmg;
    abund[s[S_NP]] = p->fp;
    abund[s[S_NF]] = p->ff;
    abund[s[S_NNA]] = p->fna;
    abund[s[S_NLI]] = p->fli;
    abund[s[S_NPAH]] = p->fpah;
    abund[s[S_NSX]] = p->fs;
    abund[s[S_NSIX]] = p->fsi;
    abund[s[S_NCLX]] = p->fcl;
    if (p->ion == 0) { abund[s[S_NC]] = p->fc; abund[s[S_NCX]] = 1.e-10; }
    else if (p->ion == 1) { abund[s[S_NC]] = p->fc * SP(0.5); abund[s[S_NCX]] = p->fc * SP(0.5); }
    else if (p->ion == 2) { abund[s[S_NC]] = 1.e-10; abund[s[S_NCX]] = p->fc; }
    abund[s[S_N18O]] = p->f18o;
    abund[s[S_N15N]] = p->f15n;
    abund[s[S_N13C]] = p->f13c;
    abund[s[S_NELEC]] = abund[s[S_NCX]] + abund[s[S_NSIX]] + abund[s[S_NSX]] + abund[s[S_NCLX]] + abund[s[S_NMGX]];
    for (int i = 0; i < neq; i++) abund[i] = abund[i] * p->metallicity;
    abund[s[S_NH]] = p->fh;
    abund[s[S_NH2]] = 0.5 * (1.0 - p->fh);
    abund[s[S_ND]] = p->fd;
    abund[s[S_NHE]] = p->fhe;
  }
  abund[n->neq - 1] = c->density;
  return 0;
}

static void chem_free(chem_t* c) {
  free(c->rate);
  free(c->vdiff);
}

/* the start-of-interval part of updateChemistry (chemistry.f90:166-203) */
static void interval_rates(chem_t* c, double* abund) {
  const orc_net* n = c->net;
  const int* s = n->sp;
  if (!c->p.freefall) abund[n->neq - 1] = c->density;
  c->h2ColToCell = c->coColToCell = c->cColToCell = 0.0;
  double cs = c->cloudSize / (double)(float)c->p.points;
  double h2col = c->h2ColToCell + 0.5 * abund[s[S_NH2]] * c->density * cs;
  double cocol = c->coColToCell + 0.5 * abund[s[S_NCO]] * c->density * cs;
  double ccol = c->cColToCell + 0.5 * abund[s[S_NC]] * c->density * cs;
  double sb = 0.0, ss = 0.0;
  for (int i = 0; i < n->n_bulk; i++) sb = i == 0 ? abund[n->bulk_list[i]] : sb + abund[n->bulk_list[i]];
  for (int i = 0; i < n->n_surface; i++) ss = i == 0 ? abund[n->surface_list[i]] : ss + abund[n->surface_list[i]];
  abund[s[S_NBULK]] = sb;
  abund[s[S_NSURFACE]] = ss;
  c->safeMantle = ss > 1e-30 ? ss : 1e-30;
  c->safeBulk = sb > 1e-30 ? sb : 1e-30;
  if (n->n_refr > 0) {
    double r = 0.0;
    for (int i = 0; i < n->n_refr; i++) r += abund[n->refr_list[i]];
    c->safeBulk = c->safeBulk - r;
  }
  double q = NUM_SITES_PER_GRAIN / (GAS_DUST_DENSITY_RATIO * c->safeBulk);
  c->blr = q < 1.0 ? q : 1.0;
  calc_rates(c, abund, c->safeMantle, h2col, cocol, ccol);
}

typedef struct {
  double* abund;     /* [neq] */
  double* abstol;    /* [neq] */
  dv_t dv;
  double currentTime, targetTime, timeInYears, abstol_factor;
  int failedIntegrationCounter;
  dv_counts cnt;
  int n_retries;
} model_t;

static void dv_alloc(dv_t* d, int n) {
  d->n = n;
  d->yh = (double*)calloc((size_t)n * 8, sizeof(double));
  d->ewt = (double*)calloc((size_t)n, sizeof(double));
  d->savf = (double*)calloc((size_t)n, sizeof(double));
  d->acor = (double*)calloc((size_t)n, sizeof(double));
  d->ftem = (double*)calloc((size_t)n, sizeof(double));
  d->wm = (double*)calloc((size_t)n * n, sizeof(double));
  d->wmj = (double*)calloc((size_t)n * n, sizeof(double));
  d->ipvt = (int*)calloc((size_t)n, sizeof(int));
}
static void dv_free(dv_t* d) {
  free(d->yh); free(d->ewt); free(d->savf); free(d->acor); free(d->ftem); free(d->wm); free(d->wmj); free(d->ipvt);
}

/* integrateODESystem (chemistry.f90:241-292) */
static int integrate_interval(model_t* m, chem_t* c) {
  const orc_net* n = c->net;
  int neq = n->neq;
  for (int i = 0; i < neq; i++) {
    m->abstol[i] = m->abstol_factor * m->abund[i];
    if (m->abstol[i] < c->p.abstol_min) m->abstol[i] = c->p.abstol_min;
  }
  m->dv.atol = m->abstol;
  m->dv.rtol = c->p.reltol;
  m->dv.mxstep = c->p.mxstep;
  m->dv.chem = c;
  int istate = dvode(&m->dv, m->abund, &m->currentTime, m->targetTime, &m->cnt);
  switch (istate) {
    case -1:
    case -4:
    case -5:
      m->targetTime = m->currentTime + (m->targetTime - m->currentTime) * SP(0.1);
      break;
    case -2:
      m->abstol_factor = m->abstol_factor * 10.0;
      break;
    case -3:
      return UCL_INT_UNRECOVERABLE_ERROR;
    case ORC_CPU_LIMIT:
      return ORC_CPU_LIMIT;
    default:
      break;
  }
  if (c->p.enforceChargeConservation) {
    double e = 0.0;
    for (int i = 0; i < n->n_ions; i++) e += m->abund[n->ions[i]];
    m->abund[n->sp[S_NELEC]] = e;
  }
  return 0;
}

/* updateChemistry (chemistry.f90:145-239) */
static int update_chemistry(model_t* m, chem_t* c) {
  const orc_net* n = c->net;
  int loop = 0, flag = 0;
  double orig = m->targetTime;
  while (m->currentTime < m->targetTime && loop < 10) {
    interval_rates(c, m->abund);
    flag = integrate_interval(m, c);
    if (flag < 0) return flag;
    for (int i = 0; i < n->neq; i++)
      if (m->abund[i] < MIN_ABUND) m->abund[i] = MIN_ABUND;
    c->density = m->abund[n->neq - 1];
    loop++;
    if (loop > 1) m->n_retries++;
  }
  if (loop == 10) flag = UCL_INT_TOO_MANY_FAILS_ERROR;
  if (fabs(orig - m->targetTime) < SP(0.001) * orig) m->failedIntegrationCounter = 0;
  else m->failedIntegrationCounter++;
  if (m->failedIntegrationCounter > 10) flag = UCL_INT_TOO_MANY_FAILS_ERROR;
  return flag;
}

static void update_target_time(model_t* m) { /* cloud.f90:39-51 */
  double ty = m->timeInYears;
  if (ty >= 1.0e6) m->targetTime = (ty + 1.0e5) * SECONDS_PER_YEAR;
  else if (ty > 10.0) {
    double om = pow(10.0, floor(log10(ty)));
    m->targetTime = ((floor(ty / om) + 1.0) * om) * SECONDS_PER_YEAR;
  } else if (ty > 0.0)
    m->targetTime = 10 * ty * SECONDS_PER_YEAR;
  else
    m->targetTime = SECONDS_PER_YEAR * 1.0e-7;
}

static void write_row(const chem_t* c, const model_t* m, double* phys, double* ab, double* rates, int row) {
  phys[0] = m->timeInYears;
  phys[1] = c->density;
  phys[2] = c->gasTemp;
  phys[3] = c->dustTemp;
  phys[4] = c->av;
  phys[5] = c->p.radfield;
  phys[6] = c->p.zeta;
  phys[7] = 1.0;
  memcpy(ab, m->abund, sizeof(double) * (size_t)c->net->nspec);
  /* ratesarray(dtime, dstep, :) = rate(:nreac) (io.f90:89-93); rate() is
   * zero before the first interval (chemistry.f90:136) */
  if (rates) {
    if (row == 0) memset(rates, 0, sizeof(double) * (size_t)c->net->nreac);
    else memcpy(rates, c->rate, sizeof(double) * (size_t)c->net->nreac);
  }
}

/* ---------------------------------------------------------------------- */
/* The collapse physics module (collapse.f90, Priestley et al. 2018): modes
 * 1 BE1.1, 2 BE4, 3 filament, 4 ambipolar.  Default-REAL literals are
 * single precision promoted (SP), 'd' literals double; integer powers by
 * the binary method (ipow_bin).  The sums run left to right, as the
 * reference's loops do. */
static const double COL_MH = 1.67262164e-24, COL_AU = 2.063e5; /* constants.f90:7,12 */

static double col_unitr(void) { /* collapse.f90:190-191 */
  return sqrt(1.38e-16 * 10 / 2 / COL_MH) * pow(2 * PI_ * 6.67e-8 * 2.2e4 * COL_MH, -0.5) / PC;
}
static double col_unitt(void) { /* collapse.f90:209-210 */
  return pow(2 * PI_ * 6.67e-8 * 2.2e4 * COL_MH, -0.5) / SECONDS_PER_YEAR;
}

static double rhofit(int mode, double r, double rho0, double r0, double a) { /* collapse.f90:178-196 */
  if (mode == 1 || mode == 2) return rho0 / (1 + pow(r * COL_AU / r0, a));
  if (mode == 3) {
    double x = r / col_unitr() / r0;
    return 2.2e4 * rho0 / pow(1 + x * x, a);
  }
  return rho0 / (1 + pow(r / 7.5e-1 / r0, a));
}

static double rho0fit(int mode, double t, double tmax) { /* collapse.f90:199-222 */
  double l;
  if (mode == 1) l = SP(61.8) * pow(tmax - t, SP(-0.01)) - SP(49.4);
  else if (mode == 2) l = SP(68.4) * pow(tmax - t, SP(-0.01)) - SP(55.7);
  else if (mode == 3) l = SP(3.54) * pow(SP(5.47) - t / col_unitt(), SP(-0.15)) - SP(2.73);
  else {
    if (t <= 6.0) return 2.0e3 + 1.7e3 * (t / 6.0 - 1.0);
    l = SP(5.3) * pow(SP(16.138) - 1e-6 * t, SP(-0.1)) - 1.0;
  }
  return pow(10.0, l);
}

static double r0fit(int mode, double t, double tmax) { /* collapse.f90:225-245 */
  double l;
  if (mode == 1) l = -(SP(28.5) * pow(tmax - t, SP(-0.01))) + SP(28.93);
  else if (mode == 2) l = -(SP(39.0) * pow(tmax - t, SP(-0.01))) + SP(38.7);
  else if (mode == 3) l = -(SP(1.34) * pow(SP(5.47) - t / col_unitt(), SP(-0.15))) + SP(1.47);
  else l = -(SP(2.57) * pow(SP(16.138) - 1e-6 * t, SP(-0.1))) + SP(1.85);
  return pow(10.0, l);
}

static double afit(int mode, double t) { /* collapse.f90:248-261 */
  if (mode == 1) return 2.4;
  if (mode == 2) return SP(1.9) + 0.5 * exp(-t / SP(1e5));
  if (mode == 3) return 2.0 - 0.5 * ipow_bin(t / col_unitt() / SP(5.47), 9);
  return SP(2.4) - SP(0.2) * ipow_bin(1e-6 * t / SP(16.138), 40);
}

static double vrfit(int mode, double r, double rmin, double vmin, double a) { /* collapse.f90:264-290 */
  double v;
  if (mode == 3) {
    double nr = r / col_unitr() - rmin;
    if (nr < 0.0) v = vmin * ((nr / rmin) * (nr / rmin) - 1);
    else v = vmin * (exp(-2.0 * a * nr) - 2 * exp(-a * nr));
    return sqrt(1.38e-16 * 10 / 2 / COL_MH) * v;
  }
  if (mode == 4) {
    double rmid = 0.5, r75 = r / 7.5e-1, nr = r75 - rmin;
    if (r75 < rmin) v = vmin * ((nr / rmin) * (nr / rmin) - 1);
    else if (r75 <= rmid) v = (vmin - a) * pow(nr / (rmid - rmin), SP(0.3)) - vmin;
    else v = a / (1.0 - rmid) * (r75 - rmid) - a;
    return 1e3 * v;
  }
  return 0.0;
}

static double rminfit(int mode, double t) { /* collapse.f90:293-321 */
  if (mode == 3) {
    double tn = t / col_unitt();
    if (tn == 0.0) return 7.2;
    if (log(tn) < 1.6) return -(SP(1.149) * tn) + SP(7.2);
    if (log(tn) < 1.674) return -(SP(9.2) * log(tn)) + SP(16.25);
    return -(SP(22.0) * log(tn)) + SP(37.65);
  }
  double t6 = 1e-6 * t;
  if (t6 <= SP(10.2)) return -(SP(0.0039) * t6) + SP(0.49);
  if (t6 <= SP(15.1)) return -(SP(0.0306) * (t6 - SP(10.2))) + SP(0.45);
  return -(SP(0.282) * (t6 - SP(15.1))) + SP(0.3);
}

static double vminfit(int mode, double t) { /* collapse.f90:324-346 */
  if (mode == 3) {
    double tn = t / col_unitt();
    if (tn == 0.0) return 0.0;
    if (log(tn) < 1.6) return SP(0.0891) * tn;
    if (log(tn) < 1.674) return SP(5.5) * log(tn) - SP(8.37);
    return SP(18.9) * log(tn) - SP(30.8);
  }
  return SP(3.44) * pow(SP(16.138) - 1e-6 * t, SP(-0.35)) - SP(0.7);
}

static double avfit(int mode, double t) { /* collapse.f90:349-378 */
  if (mode == 3) {
    double tn = t / col_unitt();
    if (tn == 0.0) return 0.4;
    if (log(tn) < 1.6) return SP(0.0101) * tn + SP(0.4);
    if (log(tn) < 1.674) return SP(0.695) * log(tn) - SP(0.663);
    return SP(2.69) * log(tn) - SP(4.0);
  }
  double t6 = 1e-6 * t;
  if (t6 <= SP(10.2)) return SP(0.143) * t6;
  return SP(0.217) * (t6 - SP(10.2)) + SP(1.46);
}

static double find_coldens(int mode, double rin, double rho0, double r0, double a, double rout) {
  /* collapse.f90:157-175 */
  const int np = 10000;
  double size = rout - rin, dr = size / np, coldens = 0.0;
  if (size <= 0.0) return coldens;
  for (int i = 1; i <= np; i++) {
    double r1 = rin + (i - 1) * dr, r2 = rin + i * dr;
    double drho = 0.5 * (rhofit(mode, r2, rho0, r0, a) + rhofit(mode, r1, rho0, r0, a));
    coldens = coldens + drho * dr * PC;
  }
  return coldens;
}

static double find_mass_in_radius(int mode, double radius, double rho0, double r0, double a) {
  /* collapse.f90:117-134 */
  const int np = 1000;
  double dr = radius / np, m = 0.0;
  for (int i = 1; i <= np; i++) {
    double drho = 0.5 * (rhofit(mode, i * dr, rho0, r0, a) + rhofit(mode, (i - 1) * dr, rho0, r0, a));
    m = m + drho * dr * ((i * dr) * (i * dr));
  }
  return m;
}

static double find_new_radius(int mode, double mass, double r, double rho0, double r0, double a) {
  /* collapse.f90:137-154; -1 if the mass is not positive or not reached in
   * 2^24 steps (the reference would return an unset value or loop on) */
  double dr = r / 1.0e4, m1 = 0.0, rad = -1.0;
  if (!(0.0 < mass)) return -1.0;
  for (int i = 1; i < (1 << 24) + 1; i++) {
    double drho = 0.5 * (rhofit(mode, i * dr, rho0, r0, a) + rhofit(mode, (i - 1) * dr, rho0, r0, a));
    m1 = m1 + drho * dr * ((i * dr) * (i * dr));
    rad = i * dr;
    if (!(m1 < mass)) return rad;
  }
  return -1.0;
}

/* The hot-core physics module (hotcore.f90): the temperature ramp of a
 * protostar of mass index m (tempa 'd' literals, tempb default REAL) and
 * its output schedule; its sublimation routine does nothing on a
 * three-phase network (hotcore.f90:82-96). */
static const double HC_TEMPA[6] = {1.927e-1, 4.8560e-2, 7.8470e-3, 9.6966e-4, 1.706e-4, 4.74e-7};
static const float HC_TEMPB[6] = {0.5339f, 0.6255f, 0.8395f, 1.085f, 1.289f, 1.98f};

static double hc_target_time(double ty) { /* hotcore.f90:50-66 */
  if (ty > 1.0e6) return (ty + 1.0e5) * SECONDS_PER_YEAR;
  if (ty > 1.0e5) return (ty + 1.0e4) * SECONDS_PER_YEAR;
  if (ty > 1.0e4) return (ty + 1000.0) * SECONDS_PER_YEAR;
  if (ty > 1000) return (ty + 100.0) * SECONDS_PER_YEAR;
  if (ty > 100) return (ty + 10.0) * SECONDS_PER_YEAR;
  if (ty > 0.0) return (ty * 10.0) * SECONDS_PER_YEAR;
  return SECONDS_PER_YEAR * 1.0e-7;
}

static double hc_temperature(int m, double T, double t, const ucl_model_params* p, double cloudSize) {
  /* hotcore.f90:70-79 for dstep = points = 1 */
  if (!(T < p->maxTemperature)) return T;
  double g = (cloudSize / (p->rout * PC)) * (double)((float)1 / (float)p->points);
  g = pow(g, -0.5);
  T = p->initialTemp + ((HC_TEMPA[m - 1] * pow(t / SECONDS_PER_YEAR, (double)HC_TEMPB[m - 1])) * g);
  if (T > p->maxTemperature) T = p->maxTemperature;
  return T;
}

static double col_target_time(double ty) { /* collapse.f90:60-72 */
  if (ty > 10000) return (ty + 1000.0) * SECONDS_PER_YEAR;
  if (ty > 1000) return (ty + 100.0) * SECONDS_PER_YEAR;
  if (ty > 0.0) return (ty * 10) * SECONDS_PER_YEAR;
  return 3.16e7 * 10.e-8;
}

/* A whole CLOUD model (solveAbundances, wrap.f90:549-697, points=1), with
 * the rows of the rates array when rates_rows is not NULL */
int orc_cloud_rates(const orc_net* n, const ucl_model_params* p, const double* start, int max_rows, double* phys,
                    double* abund_rows, int* nrows, int64_t* counters /* [9] or NULL */, double* rates_rows) {
  pthread_once(&g_tab_once, init_tables);
  g_cpu_start = thread_cpu_s();
  chem_t c;
  model_t m;
  memset(&m, 0, sizeof(m));
  int neq = n->neq;
  m.abund = (double*)calloc((size_t)neq, sizeof(double));
  m.abstol = (double*)calloc((size_t)neq, sizeof(double));
  if (chem_init(&c, n, p, m.abund, 1)) { free(m.abund); free(m.abstol); return UCL_PHYSICS_INIT_ERROR; }
  if (start) {
    memcpy(m.abund, start, sizeof(double) * (size_t)n->nspec);
    m.abund[neq - 1] = start[n->nspec];
  }
  /* collapse module: initializePhysics (collapse.f90:27-58) after the
   * core's, then initializeChemistry's abund(neq) = density */
  const int cmode = p->collapse;
  double ctmax = 0.0, crad = 0.0, cmass = 0.0;
  if (cmode != 0) {
    if (cmode < 1 || cmode > 4) {
      chem_free(&c); free(m.abund); free(m.abstol);
      *nrows = 0;
      return UCL_PHYSICS_INIT_ERROR; /* "unacceptable collapse mode" */
    }
    if (cmode == 1) ctmax = 1.175e6;
    if (cmode == 2) ctmax = 1.855e5;
    if (cmode <= 2) c.p.finalTime = SP(0.97) * ctmax;
    crad = 1 * p->rout / (double)(float)p->points;
    double rho0 = rho0fit(cmode, 0.0, ctmax), r0 = r0fit(cmode, 0.0, ctmax), a = afit(cmode, 0.0);
    c.density = rhofit(cmode, p->rin, rho0, r0, a);
    if (cmode <= 2) cmass = find_mass_in_radius(cmode, crad, rho0, r0, a);
    if (!start) m.abund[neq - 1] = c.density;
  }
  const int hmode = p->hotcore;
  if (hmode != 0 && (hmode < 1 || hmode > 6 || cmode != 0)) {
    chem_free(&c); free(m.abund); free(m.abstol);
    *nrows = 0;
    return UCL_PHYSICS_INIT_ERROR; /* tempindx out of the six masses */
  }
  const ucl_model_params* pp = &c.p;
  dv_alloc(&m.dv, neq);
  m.abstol_factor = p->abstol_factor;
  int flag = 0, row = 0;
  m.currentTime = 0.0;
  m.timeInYears = 0.0;
  if (max_rows < 1) flag = UCL_NOT_ENOUGH_TIMEPOINTS_ERROR;
  else write_row(&c, &m, phys, abund_rows, rates_rows, 0);
  row = 1;
  while (flag == 0 && ((pp->endAtFinalDensity && c.density < pp->finalDens) ||
                       (!pp->endAtFinalDensity && m.timeInYears < pp->finalTime))) {
    double told = m.currentTime;
    m.timeInYears = m.currentTime / SECONDS_PER_YEAR;
    if (cmode) m.targetTime = col_target_time(m.timeInYears);
    else if (hmode) m.targetTime = hc_target_time(m.timeInYears);
    else update_target_time(&m);
    m.currentTime = told;
    flag = update_chemistry(&m, &c);
    if (flag < 0) break;
    m.timeInYears = m.targetTime / SECONDS_PER_YEAR;
    /* coreUpdatePhysics (physics-core.f90:75-88) */
    c.coldens = c.cloudSize / (double)(float)p->points * c.density;
    c.av = p->baseAv + c.coldens / 1.6e21;
    c.dustTemp = c.gasTemp;
    if (p->cosmicRayAttenuation && p->improvedH2CRPDissociation) c.h2CRPRate = h2_crp_rate(p, c.coldens);
    if (hmode) { /* the hot-core module's updatePhysics */
      c.gasTemp = hc_temperature(hmode, c.gasTemp, m.currentTime, p, c.cloudSize);
      c.dustTemp = c.gasTemp;
    }
    if (row >= max_rows) { flag = UCL_NOT_ENOUGH_TIMEPOINTS_ERROR; break; }
    if (cmode) {
      /* the collapse module's updatePhysics (collapse.f90:76-106) */
      double t = m.timeInYears;
      double rho0 = rho0fit(cmode, t, ctmax), r0 = r0fit(cmode, t, ctmax), a = afit(cmode, t);
      c.coldens = find_coldens(cmode, p->rin, rho0, r0, a, p->rout);
      c.av = p->baseAv + c.coldens / 1.6e21;
      if (cmode <= 2) {
        crad = find_new_radius(cmode, cmass, p->rout, rho0, r0, a);
      } else {
        double dt = m.targetTime - m.currentTime; /* zero: the chemistry reached targetTime */
        crad = crad + vrfit(cmode, crad, rminfit(cmode, t), vminfit(cmode, t), avfit(cmode, t)) * dt / PC;
      }
      if (!(crad >= 0.0)) { flag = UCL_INT_UNRECOVERABLE_ERROR; break; }
      c.density = rhofit(cmode, crad, rho0, r0, a);
    }
    write_row(&c, &m, phys + (size_t)row * UCL_N_PHYS, abund_rows + (size_t)row * n->nspec,
              rates_rows ? rates_rows + (size_t)row * n->nreac : NULL, row);
    row++;
  }
  *nrows = row;
  if (counters) {
    counters[0] = m.cnt.nst; counters[1] = m.cnt.nfe; counters[2] = m.cnt.nje; counters[3] = m.cnt.nlu;
    counters[4] = m.cnt.nni; counters[5] = m.cnt.ncfn; counters[6] = m.cnt.netf; counters[7] = row;
    counters[8] = m.n_retries;
  }
  dv_free(&m.dv);
  chem_free(&c);
  free(m.abund);
  free(m.abstol);
  return flag;
}

int orc_cloud(const orc_net* n, const ucl_model_params* p, const double* start, int max_rows, double* phys,
              double* abund_rows, int* nrows, int64_t* counters /* [9] or NULL */) {
  return orc_cloud_rates(n, p, start, max_rows, phys, abund_rows, nrows, counters, NULL);
}

/* Many models on `nthreads` host threads (models are independent). */
typedef struct {
  const orc_net* n;
  const ucl_model_params* p;
  const double* start;
  int max_rows;
  double *phys, *abund;
  int *nrows, *flags;
  int64_t* counters;
  int nmodels;
  int next;
  pthread_mutex_t mu;
} batch_t;

static void* batch_worker(void* arg) {
  batch_t* b = (batch_t*)arg;
  int nspec = b->n->nspec;
  for (;;) {
    pthread_mutex_lock(&b->mu);
    int i = b->next++;
    pthread_mutex_unlock(&b->mu);
    if (i >= b->nmodels) break;
    b->flags[i] = orc_cloud(b->n, &b->p[i], b->start ? b->start + (size_t)i * (nspec + 1) : NULL, b->max_rows,
                            b->phys + (size_t)i * b->max_rows * UCL_N_PHYS,
                            b->abund + (size_t)i * b->max_rows * nspec, &b->nrows[i],
                            b->counters ? b->counters + 9 * (size_t)i : NULL);
  }
  return NULL;
}

int orc_cloud_batch(const orc_net* n, int nmodels, const ucl_model_params* p, const double* start, int max_rows,
                    double* phys, double* abund, int* nrows, int* flags, int64_t* counters, int nthreads) {
  pthread_once(&g_tab_once, init_tables);
  batch_t b = {n, p, start, max_rows, phys, abund, nrows, flags, counters, nmodels, 0, PTHREAD_MUTEX_INITIALIZER};
  if (nthreads < 1) nthreads = 1;
  pthread_t th[256];
  if (nthreads > 256) nthreads = 256;
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, batch_worker, &b);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Single-state probes used by the kernel parity tests.                  */

/* Rates at the start of the first interval for a given abundance vector
 * (the sequence updateChemistry runs before integrating).  abund [neq] is
 * updated with the refreshed surface/bulk totals.  out_phys receives
 * {av, safeMantle, bulkLayersReciprocal, phi_after}. */
int orc_rates(const orc_net* n, const ucl_model_params* p, double* abund, double phi_in, double* rates,
              double* out_phys) {
  pthread_once(&g_tab_once, init_tables);
  chem_t c;
  double* tmp = (double*)calloc((size_t)n->neq, sizeof(double));
  if (chem_init(&c, n, p, tmp, 0)) { free(tmp); return -1; }
  free(tmp);
  c.phi = phi_in;
  c.density = abund[n->neq - 1];
  int ff = c.p.freefall;
  c.p.freefall = 1; /* keep the caller's density */
  interval_rates(&c, abund);
  c.p.freefall = ff;
  memcpy(rates, c.rate, sizeof(double) * (size_t)n->nreac);
  if (out_phys) {
    out_phys[0] = c.av;
    out_phys[1] = c.safeMantle;
    out_phys[2] = c.blr;
    out_phys[3] = c.phi;
  }
  chem_free(&c);
  return 0;
}

/* F(y) for given rates (H2/CO photo rates re-evaluated from y, as F does).
 * scale [neq] (optional) receives sum |term| per row for tolerances. */
int orc_rhs(const orc_net* n, const ucl_model_params* p, const double* y, const double* rates, double* ydot,
            double* scale) {
  pthread_once(&g_tab_once, init_tables);
  chem_t c;
  double* tmp = (double*)calloc((size_t)n->neq, sizeof(double));
  if (chem_init(&c, n, p, tmp, 0)) { free(tmp); return -1; }
  free(tmp);
  memcpy(c.rate, rates, sizeof(double) * (size_t)n->nreac);
  rhs_eval(&c, y, ydot, scale);
  chem_free(&c);
  return 0;
}

/* get_odes (wrap.f90:516-547): one updateChemistry to t = 1e-7 s from the
 * given abundances, then F.  This is the path of the reference's
 * conservation known-answer test (src/uclchem/tests.py:13-66). */
int orc_get_odes(const orc_net* n, const ucl_model_params* p, const double* abund_in, double* ydot) {
  pthread_once(&g_tab_once, init_tables);
  chem_t c;
  model_t m;
  memset(&m, 0, sizeof(m));
  int neq = n->neq;
  m.abund = (double*)calloc((size_t)neq, sizeof(double));
  m.abstol = (double*)calloc((size_t)neq, sizeof(double));
  chem_init(&c, n, p, m.abund, 1);
  memcpy(m.abund, abund_in, sizeof(double) * (size_t)n->nspec);
  m.abund[neq - 1] = p->initialDens;
  dv_alloc(&m.dv, neq);
  m.abstol_factor = p->abstol_factor;
  m.currentTime = 0.0;
  m.timeInYears = 0.0;
  m.targetTime = 1.0e-7;
  int flag = update_chemistry(&m, &c);
  rhs_eval(&c, m.abund, ydot, NULL);
  dv_free(&m.dv);
  chem_free(&c);
  free(m.abund);
  free(m.abstol);
  return flag;
}

/* Finite-difference Jacobian exactly as DVJAC's MITER=2 loop forms it, at
 * state y with weights ewt_inv (1/EWT) and step h (used to cross-check the
 * analytic Jacobian of the GPU path).  jac [neq*neq] column-major. */
int orc_fd_jacobian(const orc_net* n, const ucl_model_params* p, const double* y_in, const double* rates,
                    const double* ewt_inv, double h, double* jac) {
  pthread_once(&g_tab_once, init_tables);
  chem_t c;
  int neq = n->neq;
  double* y = (double*)calloc((size_t)neq, sizeof(double));
  double* f0 = (double*)calloc((size_t)neq, sizeof(double));
  double* f1 = (double*)calloc((size_t)neq, sizeof(double));
  chem_init(&c, n, p, y, 0);
  memcpy(c.rate, rates, sizeof(double) * (size_t)n->nreac);
  memcpy(y, y_in, sizeof(double) * (size_t)neq);
  rhs_eval(&c, y, f0, NULL);
  double fac = dvnorm(neq, f0, ewt_inv);
  double r0 = 1000.0 * fabs(h) * DBL_EPSILON * (double)neq * fac;
  if (fabs(r0) <= 0.0) r0 = 1.0;
  double srur = sqrt(DBL_EPSILON);
  for (int j = 0; j < neq; j++) {
    double yj = y[j];
    double r = srur * fabs(yj), r2 = r0 / ewt_inv[j];
    if (r2 > r) r = r2;
    y[j] = y[j] + r;
    rhs_eval(&c, y, f1, NULL);
    for (int i = 0; i < neq; i++) jac[(size_t)j * neq + i] = (f1[i] - f0[i]) * (1.0 / r);
    y[j] = yj;
  }
  chem_free(&c);
  free(y); free(f0); free(f1);
  return 0;
}

/* The H2 and CO photodissociation rates F re-evaluates from y
 * (chemistry.f90:315-318). out[0] = H2, out[1] = CO. */
int orc_photo_rates(const orc_net* n, const ucl_model_params* p, const double* y, double* out) {
  pthread_once(&g_tab_once, init_tables);
  chem_t c;
  double* tmp = (double*)calloc((size_t)n->neq, sizeof(double));
  if (chem_init(&c, n, p, tmp, 0)) { free(tmp); return -1; }
  free(tmp);
  double D = y[n->neq - 1];
  double cs = c.cloudSize / (double)(float)c.p.points;
  double cocol = 0.0 + 0.5 * y[n->sp[S_NCO]] * D * cs;
  double h2col = 0.0 + 0.5 * y[n->sp[S_NH2]] * D * cs;
  out[0] = h2_photodiss_rate(h2col, c.p.radfield, c.av, 1.0);
  out[1] = co_photodiss_rate(h2col, cocol, c.p.radfield, c.av);
  chem_free(&c);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Generic mass-action systems (the synthetic networks): the same DVODE
 * (MF=22, finite-difference Jacobian, LINPACK LU) on
 *   ydot_i = sum_e coef_e * flux_{rx_e},  flux_r = k_r * y_a [* density * y_b]
 * (b < 0: one-body).  Integrated interval by interval to the output times
 * with a cold start each interval and abstol_i = max(atol_factor*y_i,
 * atol_min), the way integrateODESystem calls DVODE (chemistry.f90:241-292),
 * without UCLCHEM's retry loop.  Returns 0, or the failing ISTATE.         */
typedef struct {
  int n, m;
  const int *ra, *rb, *sptr, *srx, *scoef;
  const double* k;
  double density;
  double* flux;
} ma_t;

static void ma_rhs(void* ctx, const double* y, double* out) {
  ma_t* a = (ma_t*)ctx;
  for (int r = 0; r < a->m; r++) {
    double f = a->k[r] * y[a->ra[r]];
    if (a->rb[r] >= 0) f = f * a->density * y[a->rb[r]];
    a->flux[r] = f;
  }
  for (int i = 0; i < a->n; i++) {
    double v = 0.0;
    for (int e = a->sptr[i]; e < a->sptr[i + 1]; e++) v = v + (double)a->scoef[e] * a->flux[a->srx[e]];
    out[i] = v;
  }
}

int orc_ma_rhs(int n, int m, const int* ra, const int* rb, const double* k, double density, const int* sptr,
               const int* srx, const int* scoef, const double* y, double* ydot) {
  ma_t a = {n, m, ra, rb, sptr, srx, scoef, k, density, (double*)calloc((size_t)m, sizeof(double))};
  ma_rhs(&a, y, ydot);
  free(a.flux);
  return 0;
}

int orc_ma_solve(int n, int m, const int* ra, const int* rb, const double* k, double density, const int* sptr,
                 const int* srx, const int* scoef, double* y, int nout, const double* tout, double rtol,
                 double atol_factor, double atol_min, int mxstep, double* yout, int64_t* counts) {
  ma_t a = {n, m, ra, rb, sptr, srx, scoef, k, density, (double*)calloc((size_t)m, sizeof(double))};
  dv_t d;
  memset(&d, 0, sizeof(d));
  dv_alloc(&d, n);
  d.fn = ma_rhs;
  d.fctx = &a;
  double* atol = (double*)calloc((size_t)n, sizeof(double));
  dv_counts cnt;
  memset(&cnt, 0, sizeof(cnt));
  double t = 0.0;
  int rc = 0;
  for (int o = 0; o < nout && rc == 0; o++) {
    for (int i = 0; i < n; i++) {
      atol[i] = atol_factor * y[i];
      if (atol[i] < atol_min) atol[i] = atol_min;
    }
    d.atol = atol;
    d.rtol = rtol;
    d.mxstep = mxstep;
    const int istate = dvode(&d, y, &t, tout[o], &cnt);
    if (istate < 0) rc = istate;
    memcpy(yout + (size_t)o * n, y, sizeof(double) * (size_t)n);
  }
  if (counts) {
    counts[0] = cnt.nst; counts[1] = cnt.nfe; counts[2] = cnt.nje; counts[3] = cnt.nlu;
    counts[4] = cnt.nni; counts[5] = cnt.ncfn; counts[6] = cnt.netf;
  }
  free(atol);
  free(a.flux);
  dv_free(&d);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* A generic mass-action network integrated the way the device integrates
 * any network: NEQ = N + 1 equations with the density in the last slot
 * (zero derivative), fluxes k*D*y_a*y_b (two-body) and k*y_a (one-body),
 * and the CLOUD output schedule, retry and clamp logic of a static model
 * (cloud.f90:39-51, chemistry.f90:145-292; the same sequence as orc_cloud
 * with a constant-rate RHS).                                              */
typedef struct {
  int n, m;
  const int *ra, *rb, *sptr, *srx, *scoef;
  const double* k;
  double* flux;
} mad_t;

static void mad_rhs(void* ctx, const double* y, double* out) {
  mad_t* a = (mad_t*)ctx;
  const double D = y[a->n];
  for (int r = 0; r < a->m; r++)
    a->flux[r] = a->rb[r] >= 0 ? a->k[r] * D * y[a->ra[r]] * y[a->rb[r]] : a->k[r] * y[a->ra[r]];
  for (int i = 0; i < a->n; i++) {
    double v = 0.0;
    for (int e = a->sptr[i]; e < a->sptr[i + 1]; e++) v = v + (double)a->scoef[e] * a->flux[a->srx[e]];
    out[i] = v;
  }
  out[a->n] = 0.0;
}

int orc_ma_cloud(int n, int m, const int* ra, const int* rb, const double* k, double density, const int* sptr,
                 const int* srx, const int* scoef, const double* y0, double final_time_yr, double rtol,
                 double atol_factor, double atol_min, int mxstep, int max_rows, double* yout, double* tyr_out,
                 int* nrows, int64_t* counters /* [9] or NULL */) {
  const int neq = n + 1;
  mad_t a = {n, m, ra, rb, sptr, srx, scoef, k, (double*)calloc((size_t)m, sizeof(double))};
  model_t md;
  memset(&md, 0, sizeof(md));
  md.abund = (double*)calloc((size_t)neq, sizeof(double));
  md.abstol = (double*)calloc((size_t)neq, sizeof(double));
  memcpy(md.abund, y0, sizeof(double) * (size_t)n);
  md.abund[n] = density;
  dv_alloc(&md.dv, neq);
  md.dv.fn = mad_rhs;
  md.dv.fctx = &a;
  md.abstol_factor = atol_factor;
  int flag = 0, row = 0;
  if (max_rows < 1) flag = UCL_NOT_ENOUGH_TIMEPOINTS_ERROR;
  else {
    memcpy(yout, md.abund, sizeof(double) * (size_t)n);
    tyr_out[0] = 0.0;
    row = 1;
  }
  while (flag == 0 && md.timeInYears < final_time_yr) {
    double told = md.currentTime;
    md.timeInYears = md.currentTime / SECONDS_PER_YEAR;
    update_target_time(&md);
    md.currentTime = told;
    int loop = 0;
    double orig = md.targetTime;
    while (md.currentTime < md.targetTime && loop < 10) {
      md.abund[n] = density;
      for (int i = 0; i < neq; i++) {
        md.abstol[i] = md.abstol_factor * md.abund[i];
        if (md.abstol[i] < atol_min) md.abstol[i] = atol_min;
      }
      md.dv.atol = md.abstol;
      md.dv.rtol = rtol;
      md.dv.mxstep = mxstep;
      const int istate = dvode(&md.dv, md.abund, &md.currentTime, md.targetTime, &md.cnt);
      if (istate == -1 || istate == -4 || istate == -5)
        md.targetTime = md.currentTime + (md.targetTime - md.currentTime) * SP(0.1);
      else if (istate == -2)
        md.abstol_factor = md.abstol_factor * 10.0;
      else if (istate == -3) { flag = UCL_INT_UNRECOVERABLE_ERROR; break; }
      for (int i = 0; i < neq; i++)
        if (md.abund[i] < MIN_ABUND) md.abund[i] = MIN_ABUND;
      loop++;
      if (loop > 1) md.n_retries++;
    }
    if (flag < 0) break;
    if (loop == 10) flag = UCL_INT_TOO_MANY_FAILS_ERROR;
    if (fabs(orig - md.targetTime) < SP(0.001) * orig) md.failedIntegrationCounter = 0;
    else md.failedIntegrationCounter++;
    if (md.failedIntegrationCounter > 10) flag = UCL_INT_TOO_MANY_FAILS_ERROR;
    if (flag < 0) break;
    md.timeInYears = md.targetTime / SECONDS_PER_YEAR;
    if (row >= max_rows) { flag = UCL_NOT_ENOUGH_TIMEPOINTS_ERROR; break; }
    memcpy(yout + (size_t)row * n, md.abund, sizeof(double) * (size_t)n);
    tyr_out[row] = md.timeInYears;
    row++;
  }
  *nrows = row;
  if (counters) {
    counters[0] = md.cnt.nst; counters[1] = md.cnt.nfe; counters[2] = md.cnt.nje; counters[3] = md.cnt.nlu;
    counters[4] = md.cnt.nni; counters[5] = md.cnt.ncfn; counters[6] = md.cnt.netf; counters[7] = row;
    counters[8] = md.n_retries;
  }
  dv_free(&md.dv);
  free(md.abund);
  free(md.abstol);
  free(a.flux);
  return flag;
}
