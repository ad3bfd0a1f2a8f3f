// Host side of the C ABI (include/uclchem_gb300.h): network loading, device
// table compilation, contexts and the batched entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/uclchem_gb300.h"
#include "ucl_model.cuh"

using namespace ucl;

#define SP(x) ((double)(float)(x))

// ---------------------------------------------------------------------------
// network blob ("UCLNET01", uclchem_gb300/network.py to_blob)
struct ucl_network {
  int nspec = 0, nreac = 0, three_phase = 0;
  std::map<std::string, std::vector<int>> ints;
  std::map<std::string, std::vector<double>> dbls;
  const std::vector<int>& I(const char* k) const { return ints.at(k); }
  const std::vector<double>& D(const char* k) const { return dbls.at(k); }
};

// named-species slots in the blob's "sp" record (network.py SPECIES_PARAMS)
enum { S_NCX, S_NHX, S_NH2, S_NHE, S_NHEX, S_NN, S_NNX, S_NO, S_NOX, S_NC, S_NSIX, S_NSX, S_NH2O, S_NCH3OH,
       S_NCL, S_NCLX, S_NCO, S_NMG, S_NMGX, S_NGH, S_NGH2, S_NGN, S_NGO, S_NGOH, S_NSURFACE, S_NBULK, S_NH,
       S_ND, S_NF, S_NP, S_NS, S_NLI, S_NNA, S_NSI, S_NPAH, S_N15N, S_N13C, S_N18O, S_NELEC, S_NFE };
enum { X_H2FORM_CT, X_H2FORM_ERDES, X_H2FORM_ER, X_H2FORM_LH, X_H2FORM_LHDES, X_HFREEZE, X_EFREEZE, X_H2_HV,
       X_H2_CRP, X_H2FREEZE, X_C_HV, X_CO_HV };
enum { R_PHOTON, R_CRP, R_CRPHOT, R_FREEZE, R_DESORB, R_THERM, R_DESOH2, R_DESCR, R_DEUVCR, R_H2FORM, R_ER,
       R_ERDES, R_LH, R_LHDES, R_BULKSWAP, R_SURFSWAP, R_IONOPOL1, R_IONOPOL2, R_CRS, R_EXSOLID, R_EXRELAX,
       R_GAR, R_TWOBODY };

extern "C" int ucl_network_load(const char* path, ucl_network** out) {
  if (!path || !out) return UCL_E_ARG;
  FILE* f = fopen(path, "rb");
  if (!f) return UCL_E_NET;
  std::vector<char> buf;
  char tmp[1 << 16];
  size_t r;
  while ((r = fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
  fclose(f);
  if (buf.size() < 8 || memcmp(buf.data(), "UCLNET01", 8) != 0) return UCL_E_NET;
  ucl_network* net = new ucl_network();
  size_t off = 8;
  while (off + 44 <= buf.size()) {
    char name[33];
    memcpy(name, buf.data() + off, 32);
    name[32] = 0;
    uint32_t kind;
    uint64_t count;
    memcpy(&kind, buf.data() + off + 32, 4);
    memcpy(&count, buf.data() + off + 36, 8);
    const size_t bytes = (size_t)count * (kind == 1 ? 4 : 8);
    if (off + 44 + bytes > buf.size() || (kind != 1 && kind != 2)) { delete net; return UCL_E_NET; }
    if (kind == 1) {
      std::vector<int> v(count);
      memcpy(v.data(), buf.data() + off + 44, bytes);
      net->ints[name] = std::move(v);
    } else {
      std::vector<double> v(count);
      memcpy(v.data(), buf.data() + off + 44, bytes);
      net->dbls[name] = std::move(v);
    }
    off += 44 + bytes;
  }
  try {
    net->nspec = net->I("dims")[0];
    net->nreac = net->I("dims")[1];
    net->three_phase = net->I("dims")[2];
  } catch (...) {
    delete net;
    return UCL_E_NET;
  }
  if (net->nspec + 1 > MAX_NEQ) { delete net; return UCL_E_UNSUPPORTED; }
  *out = net;
  return UCL_OK;
}

extern "C" void ucl_network_free(ucl_network* net) { delete net; }
extern "C" int ucl_network_nspec(const ucl_network* net) { return net ? net->nspec : 0; }
extern "C" int ucl_network_nreac(const ucl_network* net) { return net ? net->nreac : 0; }

extern "C" void ucl_params_default(ucl_model_params* p) {
  memset(p, 0, sizeof(*p));
  p->initialTemp = SP(10.0); p->initialDens = 1.00e2; p->finalDens = 1.00e5; p->finalTime = 5.0e6;
  p->radfield = SP(1.0); p->zeta = SP(1.0); p->rout = SP(0.05); p->rin = SP(0.0); p->baseAv = SP(2.0);
  p->freezeFactor = SP(1.0); p->freefallFactor = SP(1.0); p->metallicity = SP(1.0);
  p->fh = SP(0.5); p->fhe = SP(0.1); p->fc = 1.77e-04; p->fo = 3.34e-04; p->fn = 6.18e-05; p->fs = 3.51e-6;
  p->fmg = 2.256e-06; p->fsi = 1.78e-06; p->fcl = 3.39e-08; p->fp = 7.78e-08; p->ff = 3.6e-08;
  p->reltol = 1e-8; p->abstol_factor = 1.0e-14; p->abstol_min = 1.0e-25;
  p->ebmaxh2 = 1.21e3; p->ebmaxcr = 1.21e3; p->ebmaxuvcr = 1.0e4; p->epsilon = SP(0.01); p->uv_yield = SP(0.03);
  p->phi = 1.0e5; p->uvcreff = 1.0e-3; p->omega = SP(0.5);
  p->desorb = p->h2desorb = p->crdesorb = p->uvdesorb = p->thermdesorb = 1;
  p->ion = 2; p->points = 1; p->mxstep = 10000;
  p->ionModel = 'L';
}

// ---------------------------------------------------------------------------
// constants and device tables
static Consts make_consts() {
  Consts K;
  memset(&K, 0, sizeof(K));
  K.K_BOLTZ = 1.38065040e-16;
  K.REDUCED_PLANCK = 1.054571628e-27;
  K.AMU = 1.66053892e-24;
  K.PI = SP(3.141592654);
  K.PC = 3.086e18;
  K.SECONDS_PER_YEAR = 3.16e7;
  K.GRAIN_RADIUS = 1.0e-5;
  K.THERMAL_VEL = sqrt(8.0 * K.K_BOLTZ / (K.PI * K.AMU));
  K.GAS_DUST_DENSITY_RATIO =
      (4.0 * K.PI * (K.GRAIN_RADIUS * K.GRAIN_RADIUS * K.GRAIN_RADIUS) * 3.0 * 100.0) / (3.0 * K.AMU);
  K.GRAIN_CROSSSECTION_PER_H = 0.5 * (7.908e-22 + 8.473e-22);
  K.GRAIN_SURFACEAREA_PER_H = 4.0 * K.GRAIN_CROSSSECTION_PER_H;
  K.SURFACE_SITE_DENSITY = 1.5e15;
  K.VDIFF_PREFACTOR = 2.0 * K.K_BOLTZ * K.SURFACE_SITE_DENSITY / K.PI / K.PI / K.AMU;
  K.NUM_SITES_PER_GRAIN = K.GRAIN_RADIUS * K.GRAIN_RADIUS * K.SURFACE_SITE_DENSITY * 4.0 * K.PI;
  K.CHEMICAL_BARRIER_THICKNESS = 1.40e-8;
  K.MAX_GRAIN_TEMP = 150.0;
  K.MIN_SURFACE_ABUND = 1.0e-20;
  K.MIN_ABUND = 1.0e-30;
  // extinction curve tau(lambda)/tau(V) (photoreactions.f90:11-24)
  const double lam[30] = {910.0, 950.0, 1000.0, 1050.0, 1110.0, 1180.0, 1250.0, 1390.0, 1490.0, 1600.0,
                          1700.0, 1800.0, 1900.0, 2000.0, 2100.0, 2190.0, 2300.0, 2400.0, 2500.0, 2740.0,
                          3440.0, 4000.0, 4400.0, 5500.0, 7000.0, 9000.0, 12500.0, 22000.0, 34000.0, 1.0e9};
  const double xl[30] = {5.76, 5.18, 4.65, 4.16, 3.73, 3.40, 3.11, 2.74, 2.63, 2.62, 2.54, 2.50, 2.58, 2.78, 3.01,
                         3.12, 2.86, 2.58, 2.35, 2.00, 1.58, 1.42, 1.32, 1.00, 0.75, 0.48, 0.28, 0.12, 0.05, 0.00};
  memcpy(K.lam, lam, sizeof(lam));
  memcpy(K.xlam, xl, sizeof(xl));
  auto natural = [](const double* x, const double* y, int n, double* y2) {
    std::vector<double> u(n);
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
    y2[n - 1] = 0.0;
    for (int k = n - 2; k >= 0; k--) y2[k] = y2[k] * y2[k + 1] + u[k];
  };
  natural(K.lam, K.xlam, 30, K.xlam_y2);
  // CO shielding table (photoreactions.f90:31-39), column by column; the
  // reference reads it through (7,6) explicit-shape dummies, so element
  // (j,k) it splines is element k*7+j of that storage sequence.
  const double sco[48] = {
      0.000e+00, -1.408e-02, -1.099e-01, -4.400e-01, -1.154e+00, -1.888e+00, -2.760e+00, -4.001e+00,
      -8.539e-02, -1.015e-01, -2.104e-01, -5.608e-01, -1.272e+00, -1.973e+00, -2.818e+00, -4.055e+00,
      -1.451e-01, -1.612e-01, -2.708e-01, -6.273e-01, -1.355e+00, -2.057e+00, -2.902e+00, -4.122e+00,
      -4.559e-01, -4.666e-01, -5.432e-01, -8.665e-01, -1.602e+00, -2.303e+00, -3.146e+00, -4.421e+00,
      -1.303e+00, -1.312e+00, -1.367e+00, -1.676e+00, -2.305e+00, -3.034e+00, -3.758e+00, -5.077e+00,
      -3.883e+00, -3.888e+00, -3.936e+00, -4.197e+00, -4.739e+00, -5.165e+00, -5.441e+00, -6.446e+00};
  for (int j = 0; j < 8; j++) K.nco_grid[j] = 12.0 + j;
  for (int k = 0; k < 6; k++) K.nh2_grid[k] = 18.0 + k;
  for (int j = 0; j < 7; j++)
    for (int k = 0; k < 6; k++) K.sco[j][k] = sco[k * 7 + j];
  for (int j = 0; j < 7; j++) natural(K.nh2_grid, K.sco[j], 6, K.sco_y2[j]);
  // column spline over the 7 N(CO) points: second derivatives are linear in
  // the values, y2 = M y; M from the same recurrence applied to unit vectors
  for (int k = 0; k < 7; k++) {
    double e[7] = {0, 0, 0, 0, 0, 0, 0}, y2[7];
    e[k] = 1.0;
    natural(K.nco_grid, e, 7, y2);
    for (int j = 0; j < 7; j++) K.sco_m[j][k] = y2[j];
  }
  K.h2_dw = 1.0 / (1000.0 * 1.0e-8);
  K.h2_r = 8.0e7 / (1.7724539 * K.h2_dw);
  K.h2_t = 3.02 * pow(K.h2_r * 1.0e+03, -0.064);
  {  // tau(1000 A)/tau(V) from the natural spline of the extinction curve
    int lo = 0, hi = 31;
    const double x = 1000.0;
    while (hi - lo != 1) { int m = (hi + lo) / 2; if (x > K.lam[m - 1]) lo = m; else hi = m; }
    if (lo == 0) { lo = 1; hi = 2; }
    if (lo == 30) { lo = 29; hi = 30; }
    const double h = K.lam[hi - 1] - K.lam[lo - 1], a = (K.lam[hi - 1] - x) / h, b = (x - K.lam[lo - 1]) / h;
    double v = a * K.xlam[lo - 1] + b * K.xlam[hi - 1] +
               ((a * a * a - a) * K.xlam_y2[lo - 1] + (b * b * b - b) * K.xlam_y2[hi - 1]) * (h * h) / 6.0;
    K.xl1000 = v < 0.0 ? 0.0 : v;
  }
  return K;
}

// host image of the device tables: every array is appended to one byte
// buffer (16-byte aligned), uploaded once, and the DevNet pointers rebased.
struct TableImage {
  std::vector<char> bytes;
  std::vector<std::pair<const void**, size_t>> fix;
  template <typename V>
  void add(const V*& field, const std::vector<V>& v) {
    size_t off = (bytes.size() + 15) / 16 * 16;
    bytes.resize(off + std::max<size_t>(v.size(), 1) * sizeof(V));
    if (!v.empty()) memcpy(bytes.data() + off, v.data(), v.size() * sizeof(V));
    fix.push_back({(const void**)&field, off});
  }
};

static double desorption_fraction(const ucl_network* net, int j, const Consts& K) {
  // chemical desorption fraction (surfacereactions.f90:218-297), a constant per reaction
  const auto& ice = net->I("ice_list");
  const auto& gice = net->I("gas_ice_list");
  const auto& re = net->I("re");
  const auto& pr = net->I("pr");
  const auto& be = net->D("binding_energy");
  const auto& fe = net->D("formation_enthalpy");
  const auto& mass = net->D("mass");
  const auto& ac = net->I("atom_counts");
  const auto& gama = net->D("gama");
  const auto& sp = net->I("sp");
  const int r1 = re[3 * j], r2 = re[3 * j + 1];
  int ri1 = 0, ri2 = 0, pi[4] = {0, 0, 0, 0};
  for (size_t i = 0; i < ice.size(); i++) {
    const int ic = ice[i], gi = gice[i];
    if (ic == r1 || gi == r1) ri1 = (int)i + 1;
    if (ic == r2 || gi == r2) ri2 = (int)i + 1;
    for (int k = 0; k < 4; k++) {
      const int p = pr[4 * j + k];
      if (p >= 0 && (ic == p || gi == p)) pi[k] = (int)i + 1;
    }
  }
  double maxbe = 0.0, ph = 0.0, eps = 0.0;
  for (int k = 0; k < 4; k++)
    if (pi[k]) {
      maxbe = std::max(maxbe, be[pi[k] - 1]);
      ph = ph + fe[pi[k] - 1];
      eps = eps + mass[pi[k] - 1];  // indexed by ice position, as the reference does
    }
  const double e = (eps - 120.0) / (eps + 120.0);
  eps = e * e;
  double dh = (ri1 ? fe[ri1 - 1] : 0.0) + (ri2 ? fe[ri2 - 1] : 0.0) - ph;
  dh = dh * 4.184e03 / (1.38054e-23 * 6.02214129e23);
  dh = dh + gama[j];
  if (dh == 0.0) dh = SP(1e-30);
  int dof = pi[0] ? ac[pi[0] - 1] : 0;
  for (int k = 1; k < 4; k++)
    if (pi[k] && ac[pi[k] - 1] > dof) dof = ac[pi[k] - 1];
  dof = 3 * dof;
  double frac = exp((-maxbe * (double)(float)dof) / (eps * dh));
  if (dh < 0.0) frac = 0.0;
  frac = frac / 10;
  const int ngn = sp[S_NGN], ngo = sp[S_NGO], ngoh = sp[S_NGOH], nh = sp[S_NH];
  if (r1 == ngn && r2 == ngn) frac = 0.5;
  if ((r1 == ngo && r2 == nh) || (r1 == nh && r2 == ngo)) frac = 0.3;
  if ((r1 == ngoh && r2 == nh) || (r1 == nh && r2 == ngoh)) frac = 0.25;
  (void)K;
  return frac;
}

struct DeviceTables {
  DevNet dn;
  void* dbuf = nullptr;
  size_t bytes = 0;
  int nchunk = 0;
  float lu_us_tc = 0.f, lu_us_cuda = 0.f;  // autotuner's FP32 LU timings (0: not measured)
};

static int build_tables(const ucl_network* net, const Consts& K, DeviceTables& T) {
  const int ns = net->nspec, nr = net->nreac, n = ns + 1;
  const auto& sp = net->I("sp");
  const auto& rx = net->I("rx");
  const auto& rg = net->I("ranges");
  const auto& re = net->I("re");
  const auto& ice = net->I("ice_list");
  const auto& surf = net->I("surface_list");
  const auto& bulk = net->I("bulk_list");
  const auto& mass = net->D("mass");
  const auto& be = net->D("binding_energy");
  const auto& alpha = net->D("alpha");
  const auto& gama = net->D("gama");
  const auto& redm = net->D("reduced_masses");
  const auto& fshape = net->I("flux_shape");
  const auto& fya = net->I("flux_ya");
  const auto& fyb = net->I("flux_yb");
  const auto& sptr = net->I("stoich_ptr");
  const auto& srx = net->I("stoich_rx");
  const auto& scoef = net->I("stoich_coef");
  const auto& swap = net->I("swap_terms");
  const int nice = (int)ice.size();
  auto range_on = [&](int r, int& a, int& b) {
    a = rg[2 * r];
    b = rg[2 * r + 1];
    return a != b && a <= nr && b <= nr;
  };
  auto ice_of = [&](int species) {
    int k = -1;
    for (int i = 0; i < nice; i++)
      if (ice[i] == species) k = i;
    return k;
  };
  auto in = [](const std::vector<int>& l, int v) { return std::find(l.begin(), l.end(), v) != l.end(); };
  std::vector<double> vdiff(nice);
  for (int i = 0; i < nice; i++) vdiff[i] = sqrt(K.VDIFF_PREFACTOR * be[i] / mass[ice[i]]);

  std::vector<uint8_t> rtype(nr, RT_NONE), iceflag(nr, 0), stick(nr, 0), extrap(nr);
  std::vector<double> c0(nr, 0.0), c1(nr, 0.0), c2(nr, 0.0), c3(nr, 0.0), c4(nr, 0.0), mre1(nr, 1.0);
  std::vector<int> partner(nr, -1), re1(nr);
  for (int j = 0; j < nr; j++) {
    re1[j] = re[3 * j];
    mre1[j] = re[3 * j] >= 0 ? mass[re[3 * j]] : 1.0;
    extrap[j] = (uint8_t)net->I("extrapolate")[j];
  }
  int a, b;
  // block order of calculateReactionRates (later blocks overwrite)
  if (range_on(R_CRP, a, b))
    for (int j = a - 1; j < b; j++) rtype[j] = RT_CRP;
  for (int blk : {R_PHOTON, R_CRPHOT})
    if (range_on(blk, a, b))
      for (int j = a - 1; j < b; j++) {
        rtype[j] = blk == R_PHOTON ? RT_PHOTON : RT_CRPHOT;
        iceflag[j] = in(bulk, re1[j]) ? 2 : in(surf, re1[j]) ? 1 : 0;
      }
  auto rx_ok = [&](int k) { return rx[k] >= 0 && rx[k] < nr; };
  if (range_on(R_FREEZE, a, b)) {
    for (int j = a - 1; j < b; j++) rtype[j] = RT_FREEZE;
    if (rx_ok(X_EFREEZE) && rx_ok(X_HFREEZE)) {
      rtype[rx[X_EFREEZE]] = RT_EFREEZE;
      partner[rx[X_EFREEZE]] = rx[X_HFREEZE];
    }
    if (rx_ok(X_H2FREEZE)) stick[rx[X_H2FREEZE]] = 1;
    if (rx_ok(X_HFREEZE)) stick[rx[X_HFREEZE]] = 2;
  }
  if (range_on(R_DESOH2, a, b))
    for (int j = a - 1; j < b; j++) rtype[j] = RT_DESOH2;
  if (range_on(R_DESCR, a, b))
    for (int j = a - 1; j < b; j++) rtype[j] = RT_DESCR;
  if (range_on(R_DEUVCR, a, b))
    for (int j = a - 1; j < b; j++) rtype[j] = RT_DEUVCR;
  if (range_on(R_CRS, a, b))
    for (int j = a - 1; j < b; j++) rtype[j] = RT_CRS;
  if (range_on(R_EXRELAX, a, b))
    for (int j = a - 1; j < b; j++) {
      const int k = ice_of(re1[j]);
      rtype[j] = RT_EXRELAX;
      c0[j] = k >= 0 ? vdiff[k] : 0.0;
    }
  if (range_on(R_EXSOLID, a, b))
    for (int j = a - 1; j < b; j++) {
      const int k1 = ice_of(re1[j]), k2 = ice_of(re[3 * j + 1]);
      rtype[j] = RT_EXSOLID;
      c0[j] = k1 >= 0 ? vdiff[k1] : 0.0;
      c1[j] = k2 >= 0 ? vdiff[k2] : 0.0;
    }
  if (range_on(R_THERM, a, b))
    for (int j = a - 1; j < b; j++) {
      const int k = ice_of(re1[j]);
      if (k >= 0) { rtype[j] = RT_THERM; c0[j] = vdiff[k]; }
    }
  if (range_on(R_LH, a, b)) {
    int d1 = rg[2 * R_LHDES], d2 = rg[2 * R_LHDES + 1];
    for (int j = a - 1; j < b; j++) {
      const int k1 = ice_of(re1[j]), k2 = ice_of(re[3 * j + 1]);
      if (k1 < 0 || k2 < 0) return UCL_E_NET;
      rtype[j] = RT_LH;
      c0[j] = vdiff[k1];
      c1[j] = vdiff[k2];
      c2[j] = be[k1];
      c3[j] = be[k2];
      double rm = redm[j];
      if (rm == 0.0) rm = mass[ice[k1]] * mass[ice[k2]] / (mass[ice[k1]] + mass[ice[k2]]);
      c4[j] = 2.0 * K.CHEMICAL_BARRIER_THICKNESS / K.REDUCED_PLANCK * sqrt(2.0 * K.AMU * rm * K.K_BOLTZ * gama[j]);
      const int jd = d1 - 1 + (j - (a - 1));
      partner[j] = (jd < d2) ? jd : -1;
    }
    for (int j = d1 - 1; j < d2; j++) {
      rtype[j] = RT_LHDES;
      partner[j] = a - 1 + (j - (d1 - 1));
      c0[j] = desorption_fraction(net, j, K);
      iceflag[j] = in(bulk, re1[j]) ? 1 : 0;
    }
  }
  if (range_on(R_ER, a, b)) {
    int d1 = rg[2 * R_ERDES], d2 = rg[2 * R_ERDES + 1];
    for (int j = a - 1; j < b; j++) {
      rtype[j] = RT_ER;
      const int jd = d1 - 1 + (j - (a - 1));
      partner[j] = (jd < d2) ? jd : -1;
    }
    for (int j = d1 - 1; j < d2; j++) {
      rtype[j] = RT_ERDES;
      partner[j] = a - 1 + (j - (d1 - 1));
      c0[j] = desorption_fraction(net, j, K);
      iceflag[j] = in(bulk, re1[j]) ? 1 : 0;
    }
  }
  if (rx_ok(X_H2FORM_CT)) rtype[rx[X_H2FORM_CT]] = RT_H2FORM;
  if (rx_ok(X_H2FORM_ER)) rtype[rx[X_H2FORM_ER]] = RT_ZERO;
  if (rx_ok(X_H2FORM_ERDES)) rtype[rx[X_H2FORM_ERDES]] = RT_ZERO;
  if (net->three_phase) {
    a = rg[2 * R_BULKSWAP];
    b = rg[2 * R_BULKSWAP + 1];
    if (a <= nr)
      for (int j = a - 1; j < b; j++) {
        const int k = ice_of(re1[j]);
        if (k >= 0) { rtype[j] = RT_BULKSWAP; c0[j] = vdiff[k]; c1[j] = be[k]; }
        else rtype[j] = RT_NONE;
      }
    a = rg[2 * R_SURFSWAP];
    b = rg[2 * R_SURFSWAP + 1];
    if (a <= nr)
      for (int j = a - 1; j < b; j++) rtype[j] = RT_SURFSWAP;
  }
  a = rg[2 * R_TWOBODY];
  b = rg[2 * R_TWOBODY + 1];
  if (a <= nr)
    for (int j = a - 1; j < b; j++) rtype[j] = RT_TWOBODY;
  if (range_on(R_IONOPOL1, a, b))
    for (int j = a - 1; j < b; j++) rtype[j] = RT_IONOPOL1;
  if (range_on(R_IONOPOL2, a, b))
    for (int j = a - 1; j < b; j++) rtype[j] = RT_IONOPOL2;
  std::vector<double> gar = net->D("gar_params");
  if (range_on(R_GAR, a, b))
    for (int j = a - 1; j < b; j++) { rtype[j] = RT_GAR; partner[j] = j - (a - 1); }
  // freeze partners
  const auto& fpv = net->I("freeze_partners");
  std::vector<int> fp(fpv.begin(), fpv.end()), fp_re1(fp.size());
  for (size_t k = 0; k < fp.size(); k++) fp_re1[k] = re1[fp[k]];
  auto first_of = [&](int blk) { int x, y; return range_on(blk, x, y) ? x - 1 : -1; };

  DevNet& D = T.dn;
  memset(&D, 0, sizeof(D));
  D.nspec = ns; D.neq = n; D.nreac = nr; D.three_phase = net->three_phase;
  D.n_surface = (int)surf.size(); D.n_bulk = (int)bulk.size(); D.n_ice = nice;
  D.nh = sp[S_NH]; D.nh2 = sp[S_NH2]; D.nhe = sp[S_NHE]; D.nc = sp[S_NC]; D.ncx = sp[S_NCX]; D.nco = sp[S_NCO];
  D.nelec = sp[S_NELEC]; D.nsurf = sp[S_NSURFACE]; D.nbulk = sp[S_NBULK]; D.nmgx = sp[S_NMGX];
  D.nsix = sp[S_NSIX]; D.nsx = sp[S_NSX]; D.nclx = sp[S_NCLX]; D.no = sp[S_NO]; D.nn = sp[S_NN];
  D.nmg = sp[S_NMG]; D.np = sp[S_NP]; D.nf = sp[S_NF]; D.nna = sp[S_NNA]; D.nli = sp[S_NLI];
  D.npah = sp[S_NPAH]; D.nd = sp[S_ND]; D.n18o = sp[S_N18O]; D.n15n = sp[S_N15N]; D.n13c = sp[S_N13C];
  D.rx_h2hv = rx_ok(X_H2_HV) ? rx[X_H2_HV] : -1;
  D.rx_cohv = rx_ok(X_CO_HV) ? rx[X_CO_HV] : -1;
  D.rx_chv = rx_ok(X_C_HV) ? rx[X_C_HV] : -1;
  D.rx_h2crp = rx_ok(X_H2_CRP) ? rx[X_H2_CRP] : -1;
  // ion list (chemistry.f90:114-121: species whose name contains '+'), and
  // the refractory list (chemistry.f90:196); older blobs carry neither
  std::vector<int> ions, refr;
  if (net->ints.count("ion_list")) ions = net->I("ion_list");
  if (net->ints.count("refractory_list")) refr = net->I("refractory_list");
  for (int i : ions)
    if (i < 0 || i >= ns) return UCL_E_NET;
  for (int i : refr)
    if (i < 0 || i >= ns) return UCL_E_NET;
  D.n_ion = (int)ions.size();
  D.n_refr = (int)refr.size();
  // linear invariants [E][nspec] (older blobs: none, no projection)
  std::vector<int> isp_ptr(n + 1, 0), iel_ptr(1, 0);
  std::vector<unsigned> isp, iel;
  if (net->ints.count("inv_counts")) {
    const auto& ic = net->I("inv_counts");
    if (ic.size() % ns != 0) return UCL_E_NET;
    const int E = (int)(ic.size() / ns);
    if (E <= MAX_INV) {
      for (int e = 0; e < E; ++e) {
        for (int i = 0; i < ns; ++i) {
          const int cnt = ic[(size_t)e * ns + i];
          if (cnt < -128 || cnt > 127) return UCL_E_NET;
          if (cnt) iel.push_back((unsigned)i << 8 | ((unsigned)cnt & 0xFFu));
        }
        iel_ptr.push_back((int)iel.size());
      }
      for (int i = 0; i < ns; ++i) {
        for (int e = 0; e < E; ++e) {
          const int cnt = ic[(size_t)e * ns + i];
          if (cnt) isp.push_back((unsigned)e << 8 | ((unsigned)cnt & 0xFFu));
        }
        isp_ptr[i + 1] = (int)isp.size();
      }
      isp_ptr[n] = (int)isp.size();
      D.n_inv = E;
    }
  }
  D.n_fp = (int)fp.size();
  D.desoh2_1 = first_of(R_DESOH2); D.descr_1 = first_of(R_DESCR); D.deuvcr_1 = first_of(R_DEUVCR);
  D.therm_1 = first_of(R_THERM);
  // flux form
  std::vector<uint8_t> fsh(nr);
  for (int j = 0; j < nr; j++) {
    if (fshape[j] < 0) return UCL_E_NET;
    fsh[j] = (uint8_t)fshape[j];
  }
  a = rg[2 * R_BULKSWAP];
  b = rg[2 * R_BULKSWAP + 1];
  if (a > nr || b > nr || a > b) { a = 1; b = 0; }  // no bulk-swap reactions
  D.swap_lo = a - 1;
  D.swap_hi = b;
  {  // totalSwap must be the sum of the bulk-swap fluxes
    const int nsw = (int)swap.size() / 2;
    if (nsw != b - a + 1) return UCL_E_NET;
    for (int k = 0; k < nsw; k++)
      if (swap[2 * k] != a - 1 + k || fsh[swap[2 * k]] != SH_Y_BLR) return UCL_E_NET;
  }
  std::vector<int> ts;
  for (int j = 0; j < nr; j++)
    if (fsh[j] == SH_Y_TS_SM) ts.push_back(j);
  D.n_ts = (int)ts.size();
  // chunked CSR of species rows (all rows but the SURFACE/BULK totals)
  const int CH = 12;
  std::vector<int> ch_row, ch_beg, ch_end;
  for (int i = 0; i < ns; i++) {
    if (i == D.nsurf || i == D.nbulk) continue;
    int s0 = sptr[i], s1 = sptr[i + 1];
    if (s0 == s1) { ch_row.push_back(i); ch_beg.push_back(s0); ch_end.push_back(s1); }
    for (int s = s0; s < s1; s += CH) {
      ch_row.push_back(i);
      ch_beg.push_back(s);
      ch_end.push_back(std::min(s + CH, s1));
    }
  }
  D.nchunk = (int)ch_row.size();
  T.nchunk = D.nchunk;
  std::vector<float> st_coef(scoef.begin(), scoef.end());
  // packed forms (field widths checked)
  std::vector<unsigned> fpack(nr), chpack(D.nchunk), stpack(srx.size()), rowch(n, 0u);
  for (int j = 0; j < nr; j++) {
    if (fya[j] < 0 || fya[j] >= 0x3FFF || fyb[j] + 1 >= 0x3FFF || fsh[j] >= 16) return UCL_E_NET;
    fpack[j] = (unsigned)fsh[j] << 28 | (unsigned)(fyb[j] + 1) << 14 | (unsigned)fya[j];
  }
  if (srx.size() >= 0x10000 || D.nchunk >= 0x10000 || n >= 1024) return UCL_E_NET;
  for (int c = 0; c < D.nchunk; c++) {
    chpack[c] = (unsigned)ch_row[c] << 20 | (unsigned)(ch_end[c] - ch_beg[c]) << 16 | (unsigned)ch_beg[c];
    if (c == 0 || ch_row[c - 1] != ch_row[c]) rowch[ch_row[c]] = (unsigned)c;
    rowch[ch_row[c]] += 1u << 16;
  }
  for (size_t e = 0; e < srx.size(); e++) {
    if (scoef[e] < -128 || scoef[e] > 127 || srx[e] >= 0x10000) return UCL_E_NET;
    stpack[e] = ((unsigned)scoef[e] & 0xFFu) << 16 | (unsigned)srx[e];
  }
  // stoichiometric coefficient lookup per (row, reaction) incl. the SURFACE total
  std::vector<std::map<int, int>> rowc(n);
  for (int i = 0; i < ns; i++)
    for (int s = sptr[i]; s < sptr[i + 1]; s++) rowc[i][srx[s]] += scoef[s];
  for (int k : surf)
    for (auto& kv : rowc[k]) rowc[D.nsurf][kv.first] += kv.second;
  // Jacobian structural entries
  static const int dpow[10] = {1, 0, 1, 0, 0, 0, 0, 1, 0, 1};
  static const int has_b[10] = {1, 0, 0, 0, 1, 1, 0, 1, 0, 1};
  static const int has_sm[10] = {0, 0, 0, 1, 0, 0, 0, 1, 1, 1};
  static const int has_blr[10] = {0, 0, 0, 0, 0, 1, 1, 0, 1, 0};
  std::map<std::pair<int, int>, std::vector<std::pair<int, float>>> ent;
  for (int i = 0; i < n; i++) {
    if (i == D.nbulk) continue;
    for (auto& kv : rowc[i]) {
      const int r = kv.first;
      const float c = (float)kv.second;
      if (kv.second == 0) continue;
      const int sh = fsh[r];
      ent[{i, fya[r]}].push_back({r << 3 | 0, c});
      if (has_b[sh]) ent[{i, fyb[r]}].push_back({r << 3 | 1, c});
      if (dpow[sh]) ent[{i, n - 1}].push_back({r << 3 | 2, c});
      if (has_sm[sh]) ent[{i, D.nsurf}].push_back({r << 3 | 3, c});
      if (has_blr[sh]) ent[{i, D.nbulk}].push_back({r << 3 | 4, c});
    }
  }
  std::vector<int> je_row, je_col, je_beg, je_end, jc_key;
  std::vector<float> jc_coef;
  for (auto& kv : ent) {
    je_row.push_back(kv.first.first);
    je_col.push_back(kv.first.second);
    je_beg.push_back((int)jc_key.size());
    for (auto& c : kv.second) { jc_key.push_back(c.first); jc_coef.push_back(c.second); }
    je_end.push_back((int)jc_key.size());
  }
  D.n_jent = (int)je_row.size();
  // the same entries as chunks of <= 8 contributions (a few entries, e.g. the
  // density column, have hundreds), packed one word per item:
  //   jent[e]  = nchunks << 16 | first chunk
  //   jchunk[c] = len << 16 | first contribution
  //   jcpack[k] = (coef & 0xff) << 16 | (reaction << 3 | slot)
  std::vector<unsigned> jent, jchunk, jcpack;
  {
    const int JCH = 8;
    if (jc_key.size() >= 0x10000) return UCL_E_NET;
    for (size_t e = 0; e < je_row.size(); e++) {
      const unsigned first = (unsigned)jchunk.size();
      for (int b = je_beg[e]; b < je_end[e]; b += JCH)
        jchunk.push_back((unsigned)std::min(JCH, je_end[e] - b) << 16 | (unsigned)b);
      jent.push_back(((unsigned)jchunk.size() - first) << 16 | first);
    }
    if (jchunk.size() >= 0x10000) return UCL_E_NET;
    for (size_t k = 0; k < jc_key.size(); k++) {
      const int cf = (int)jc_coef[k];
      if ((float)cf != jc_coef[k] || cf < -128 || cf > 127 || jc_key[k] >= 0x10000) return UCL_E_NET;
      jcpack.push_back(((unsigned)cf & 0xFFu) << 16 | (unsigned)jc_key[k]);
    }
  }
  D.njch = (int)jchunk.size();
  D.npart = std::max(D.nchunk, D.njch);
  T.nchunk = D.nchunk;
  // surface-swap rank-1 rows
  std::vector<int> ar_row, ar_beg, ar_end, ar_rx;
  std::vector<float> ar_coef;
  for (int i = 0; i < n; i++) {
    if (i == D.nbulk) continue;
    std::vector<std::pair<int, int>> l;
    for (int r : ts) {
      auto it = rowc[i].find(r);
      if (it != rowc[i].end() && it->second != 0) l.push_back({r, it->second});
    }
    if (l.empty()) continue;
    ar_row.push_back(i);
    ar_beg.push_back((int)ar_rx.size());
    for (auto& p : l) { ar_rx.push_back(p.first); ar_coef.push_back((float)p.second); }
    ar_end.push_back((int)ar_rx.size());
  }
  D.n_arow = (int)ar_row.size();
  // photo rows
  std::vector<int> ph_row;
  std::vector<float> ph_c1, ph_c2;
  for (int i = 0; i < n; i++) {
    if (i == D.nbulk || i == D.nsurf) continue;
    auto f1 = rowc[i].find(D.rx_h2hv);
    auto f2 = rowc[i].find(D.rx_cohv);
    const int c1v = f1 != rowc[i].end() ? f1->second : 0, c2v = f2 != rowc[i].end() ? f2->second : 0;
    if (c1v == 0 && c2v == 0) continue;
    ph_row.push_back(i);
    ph_c1.push_back((float)c1v);
    ph_c2.push_back((float)c2v);
  }
  D.n_ph = (int)ph_row.size();
  if (D.n_ph > NT || D.n_arow > 1000 - 0) return UCL_E_UNSUPPORTED;
  if ((D.rx_h2hv >= 0 && fsh[D.rx_h2hv] != SH_Y) || (D.rx_cohv >= 0 && fsh[D.rx_cohv] != SH_Y))
    return UCL_E_UNSUPPORTED;
  if (sp[S_NSURFACE] != ns - 1 - 0 && false) return UCL_E_NET;

  // upload
  TableImage img;
  std::vector<int> surfv(surf.begin(), surf.end()), bulkv(bulk.begin(), bulk.end());
  img.add(D.surface_list, surfv);
  img.add(D.bulk_list, bulkv);
  img.add(D.rtype, rtype);
  img.add(D.iceflag, iceflag);
  img.add(D.re1, re1);
  img.add(D.alpha, alpha);
  img.add(D.beta, net->D("beta"));
  img.add(D.gama, gama);
  img.add(D.tmin, net->D("min_temps"));
  img.add(D.tmax, net->D("max_temps"));
  img.add(D.extrap, extrap);
  img.add(D.mass_re1, mre1);
  img.add(D.c0, c0);
  img.add(D.c1, c1);
  img.add(D.c2, c2);
  img.add(D.c3, c3);
  img.add(D.c4, c4);
  img.add(D.partner, partner);
  img.add(D.stick, stick);
  img.add(D.gar, gar);
  img.add(D.fp, fp);
  img.add(D.fp_re1, fp_re1);
  img.add(D.fshape, fsh);
  std::vector<int> fyav(fya.begin(), fya.end()), fybv(fyb.begin(), fyb.end());
  img.add(D.fya, fyav);
  img.add(D.fyb, fybv);
  img.add(D.ts_rx, ts);
  img.add(D.ch_row, ch_row);
  img.add(D.ch_beg, ch_beg);
  img.add(D.ch_end, ch_end);
  std::vector<int> srxv(srx.begin(), srx.end());
  img.add(D.st_rx, srxv);
  img.add(D.st_coef, st_coef);
  img.add(D.fpack, fpack);
  img.add(D.chpack, chpack);
  img.add(D.stpack, stpack);
  img.add(D.rowch, rowch);
  img.add(D.je_row, je_row);
  img.add(D.je_col, je_col);
  img.add(D.je_beg, je_beg);
  img.add(D.je_end, je_end);
  img.add(D.jc_key, jc_key);
  img.add(D.jc_coef, jc_coef);
  img.add(D.jent, jent);
  img.add(D.jchunk, jchunk);
  img.add(D.jcpack, jcpack);
  img.add(D.ar_row, ar_row);
  img.add(D.ar_beg, ar_beg);
  img.add(D.ar_end, ar_end);
  img.add(D.ar_rx, ar_rx);
  img.add(D.ar_coef, ar_coef);
  img.add(D.ion_list, ions);
  img.add(D.refr_list, refr);
  img.add(D.inv_sp_ptr, isp_ptr);
  img.add(D.inv_sp, isp);
  img.add(D.inv_el_ptr, iel_ptr);
  img.add(D.inv_el, iel);
  img.add(D.ph_row, ph_row);
  img.add(D.ph_c1, ph_c1);
  img.add(D.ph_c2, ph_c2);
  if (cudaMalloc(&T.dbuf, img.bytes.size()) != cudaSuccess) return UCL_E_NOMEM;
  if (cudaMemcpy(T.dbuf, img.bytes.data(), img.bytes.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(T.dbuf);
    return UCL_E_CUDA;
  }
  for (auto& fx : img.fix) *fx.first = (const char*)T.dbuf + fx.second;
  T.bytes = img.bytes.size();
  return UCL_OK;
}

// ---------------------------------------------------------------------------
// context
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return UCL_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return UCL_E_NOMEM;
    cap = bytes;
    return UCL_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct ucl_ctx {
  int device = 0;
  int nsm = 0;
  size_t budget = 0;
  cudaStream_t stream = nullptr;
  std::vector<DeviceTables> tabs;  // one per network of the context
  DevNet* nets_d = nullptr;        // device copy of every tabs[k].dn
  // largest NEQ-1 / NEQ / reactions over the networks: the per-model strides
  // of every batched array and the size of the per-slot workspace
  int nspec = 0, nreac = 0, neq = 0;
  int njch = 0;                    // largest Jacobian chunk count (per-slot partial sums)
  size_t smem32 = 0, smem64 = 0;   // solver shared memory for the largest need
  DevBuf ws, io, small;
  int slots_fp32 = 0, slots_fp64 = 0;
};

template <typename T>
static size_t slot_bytes(int n, int nreac, int njch) {
  return (size_t)nreac * 8 + 2 * mat_stride(n) * sizeof(T) + (size_t)n * 4 +
         (size_t)2 * LuCfg<T>::NB * n * sizeof(T) + dinv_elems(n) * sizeof(T) + (size_t)njch * 8 +
         (size_t)MAX_INV * MAX_INV * 8 + 7 * 256;
}

template <typename T>
static size_t solver_smem(const ucl_ctx* c) {
  size_t m = 0;
  for (const auto& t : c->tabs) m = std::max(m, smem_layout<T>(t.dn.neq, t.dn.nreac, t.dn.nchunk).total);
  return m;
}

template <typename T>
static int max_slots(ucl_ctx* c) {
  const size_t sm = sizeof(T) == 4 ? c->smem32 : c->smem64;
  if (cudaFuncSetAttribute(k_solve_models<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
      cudaSuccess)
    return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_models<T>, NT, sm) != cudaSuccess)
    return 0;
  // make sure the per-thread stack covers the kernel's static local memory
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, k_solve_models<T>) == cudaSuccess) {
    size_t cur = 0;
    cudaDeviceGetLimit(&cur, cudaLimitStackSize);
    const size_t need = (fa.localSizeBytes + 1023) / 1024 * 1024 + 1024;
    if (cur < need) cudaDeviceSetLimit(cudaLimitStackSize, need);
  }
  return per_sm * c->nsm;
}

// LU-variant autotuner.  Per network, time the FP32 factorisation of a wave
// of Newton-like test matrices (I - R, R random with column scales
// 10^U(-3,1), a fixed seed) with the tensor-core and with the CUDA-core
// trailing update, and keep the faster for that network's solves
// (DevNet::lu_tc).  Networks above TC_MAX_N have only the CUDA-core update.
// UCL_AUTOTUNE=0 in the environment skips the timing and keeps the tensor
// cores wherever they apply.
static int tune_lu(ucl_ctx* c, DeviceTables& t) {
  const int n = t.dn.neq;
  t.dn.lu_tc = LuSmem<float>::tc_ok(n) ? 1 : 0;
  const char* env = getenv("UCL_AUTOTUNE");
  if (!t.dn.lu_tc || (env && env[0] == '0')) return UCL_OK;
  const int B = std::min(32, std::max(1, c->nsm));
  const size_t nn = (size_t)n * n;
  std::vector<float> h(nn * B);
  uint64_t st = 0x9E3779B97F4A7C15ull ^ (uint64_t)n;
  auto next = [&st]() {  // splitmix64
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int b = 0; b < B; ++b) {
    std::vector<double> cs(n);
    for (int j = 0; j < n; ++j) cs[j] = pow(10.0, -3.0 + 4.0 * next());
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        h[b * nn + (size_t)i * n + j] = (float)((i == j ? 1.0 : 0.0) - (2.0 * next() - 1.0) * cs[j]);
  }
  float *src = nullptr, *work = nullptr, *scr = nullptr;
  int *perm = nullptr, *info = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = UCL_E_CUDA;
  const size_t sm = lu_smem_bytes<float>(n);
  do {
    if (cudaMalloc(&src, nn * B * 4) != cudaSuccess || cudaMalloc(&work, nn * B * 4) != cudaSuccess ||
        cudaMalloc(&scr, (size_t)B * 2 * LuCfg<float>::NB * n * 4) != cudaSuccess ||
        cudaMalloc(&perm, (size_t)B * n * 4) != cudaSuccess || cudaMalloc(&info, (size_t)B * 4) != cudaSuccess) {
      rc = UCL_E_NOMEM;
      break;
    }
    if (cudaMemcpy(src, h.data(), nn * B * 4, cudaMemcpyHostToDevice) != cudaSuccess) break;
    if (cudaFuncSetAttribute(k_lu_batch<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
        cudaSuccess)
      break;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) break;
    float best[2] = {1e30f, 1e30f};
    bool ok = true;
    for (int rep = 0; rep < 3 && ok; ++rep)
      for (int v = 0; v < 2 && ok; ++v) {  // v = 1: tensor cores
        ok = cudaMemcpyAsync(work, src, nn * B * 4, cudaMemcpyDeviceToDevice, c->stream) == cudaSuccess &&
             cudaEventRecord(e0, c->stream) == cudaSuccess;
        k_lu_batch<float><<<B, NT, sm, c->stream>>>(work, n, perm, info, scr, B, v);
        ok = ok && cudaGetLastError() == cudaSuccess && cudaEventRecord(e1, c->stream) == cudaSuccess &&
             cudaEventSynchronize(e1) == cudaSuccess;
        float ms = 0.f;
        ok = ok && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
        if (ok) best[v] = std::min(best[v], ms * 1e3f);
      }
    if (!ok) break;
    t.lu_us_cuda = best[0];
    t.lu_us_tc = best[1];
    t.dn.lu_tc = best[1] <= best[0] ? 1 : 0;
    rc = UCL_OK;
  } while (false);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(src);
  cudaFree(work);
  cudaFree(scr);
  cudaFree(perm);
  cudaFree(info);
  return rc;
}

static void ctx_free(ucl_ctx* c) {
  for (auto& t : c->tabs) cudaFree(t.dbuf);
  if (c->nets_d) cudaFree(c->nets_d);
  if (c->stream) cudaStreamDestroy(c->stream);
  c->ws.release();
  c->io.release();
  c->small.release();
  delete c;
}

static int ctx_create(const ucl_network* const* nets, int nnets, int device, size_t hbm_budget, ucl_ctx** out) {
  if (!nets || nnets < 1 || !out) return UCL_E_ARG;
  for (int k = 0; k < nnets; ++k)
    if (!nets[k]) return UCL_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return UCL_E_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return UCL_E_CUDA;
  ucl_ctx* c = new ucl_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  c->budget = hbm_budget ? hbm_budget : ((size_t)8 << 30);
  const Consts K = make_consts();
  if (cudaMemcpyToSymbol(cK, &K, sizeof(K)) != cudaSuccess) { ctx_free(c); return UCL_E_CUDA; }
  for (int k = 0; k < nnets; ++k) {
    c->tabs.emplace_back();
    const int rc = build_tables(nets[k], K, c->tabs.back());
    if (rc != UCL_OK) {
      c->tabs.pop_back();
      ctx_free(c);
      return rc;
    }
    c->nspec = std::max(c->nspec, nets[k]->nspec);
    c->nreac = std::max(c->nreac, nets[k]->nreac);
    c->njch = std::max(c->njch, c->tabs.back().dn.njch);
  }
  c->neq = c->nspec + 1;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { ctx_free(c); return UCL_E_CUDA; }
  for (auto& t : c->tabs) {
    const int rc = tune_lu(c, t);
    if (rc != UCL_OK) { ctx_free(c); return rc; }
  }
  std::vector<DevNet> dn;
  for (const auto& t : c->tabs) dn.push_back(t.dn);
  if (cudaMalloc(&c->nets_d, dn.size() * sizeof(DevNet)) != cudaSuccess) { ctx_free(c); return UCL_E_NOMEM; }
  if (cudaMemcpy(c->nets_d, dn.data(), dn.size() * sizeof(DevNet), cudaMemcpyHostToDevice) != cudaSuccess) {
    ctx_free(c);
    return UCL_E_CUDA;
  }
  c->smem32 = solver_smem<float>(c);
  c->smem64 = solver_smem<double>(c);
  c->slots_fp32 = max_slots<float>(c);
  c->slots_fp64 = max_slots<double>(c);
  if (!c->slots_fp32 || !c->slots_fp64) { ctx_free(c); return UCL_E_UNSUPPORTED; }
  *out = c;
  return UCL_OK;
}

extern "C" int ucl_ctx_create(const ucl_network* net, int device, size_t hbm_budget, ucl_ctx** out) {
  return ctx_create(&net, 1, device, hbm_budget, out);
}

extern "C" int ucl_ctx_create_multi(const ucl_network* const* nets, int nnets, int device, size_t hbm_budget,
                                    ucl_ctx** out) {
  return ctx_create(nets, nnets, device, hbm_budget, out);
}

extern "C" void ucl_ctx_destroy(ucl_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  ctx_free(c);
}

static int cuda_status(cudaError_t e) { return e == cudaSuccess ? UCL_OK : UCL_E_CUDA; }

// a SolveIO with the context's strides; the caller fills the arrays
static SolveIO make_io(const ucl_ctx* c, int nmodels, int max_rows) {
  SolveIO io;
  memset(&io, 0, sizeof(io));
  io.nmodels = nmodels;
  io.max_rows = max_rows;
  io.start_stride = c->neq;
  io.ab_stride = c->nspec;
  io.rate_stride = c->nreac;
  io.nets = c->nets_d;
  return io;
}

// ---------------------------------------------------------------------------
// device-pointer solve (inputs already resident on the device)
template <typename T>
static int solve_dev(ucl_ctx* c, DevBuf& wsbuf, const SolveIO& io, int nslots_req, cudaStream_t st,
                     const double* arrival_d = nullptr, LiveQueue q = LiveQueue{}) {
  const int n = c->neq, nmodels = io.nmodels;
  int nslots = sizeof(T) == 4 ? c->slots_fp32 : c->slots_fp64;
  if (nslots_req > 0) nslots = std::min(nslots, nslots_req);
  const size_t per = slot_bytes<T>(n, c->nreac, c->njch);
  nslots = (int)std::min<size_t>(nslots, std::max<size_t>(1, c->budget / per));
  nslots = std::min(nslots, nmodels);
  if (nslots < 1) return UCL_OK;
  // every region 256-byte aligned (the LU uses 16-byte vector accesses)
  auto a256 = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t yh_b = 256, rate_b = a256((size_t)nslots * c->nreac * 8),
               j_b = a256((size_t)nslots * mat_stride(n) * sizeof(T)), perm_b = a256((size_t)nslots * n * 4),
               scr_b = a256((size_t)nslots * 2 * LuCfg<T>::NB * n * sizeof(T)),
               dinv_b = a256((size_t)nslots * dinv_elems(n) * sizeof(T)),
               jp_b = a256((size_t)nslots * c->njch * 8),
               gi_b = a256((size_t)nslots * MAX_INV * MAX_INV * 8);
  const size_t order_b = a256((size_t)nmodels * 4);
  int rc = wsbuf.ensure(yh_b + rate_b + 2 * j_b + perm_b + scr_b + dinv_b + jp_b + gi_b + 512 + order_b);
  if (rc) return rc;
  char* base = (char*)wsbuf.p;
  SlotArrays<T> A;
  A.yh = (double*)base;
  A.rate = (double*)(base + yh_b);
  A.J = (T*)(base + yh_b + rate_b);
  A.P = (T*)(base + yh_b + rate_b + j_b);
  A.perm = (int*)(base + yh_b + rate_b + 2 * j_b);
  A.scr = (T*)(base + yh_b + rate_b + 2 * j_b + perm_b);
  A.dinv = (T*)(base + yh_b + rate_b + 2 * j_b + perm_b + scr_b);
  A.jpart = (double*)(base + yh_b + rate_b + 2 * j_b + perm_b + scr_b + dinv_b);
  A.ginv = (double*)(base + yh_b + rate_b + 2 * j_b + perm_b + scr_b + dinv_b + jp_b);
  A.n = n;
  A.nreac = c->nreac;
  A.njch = c->njch;
  int* counter = (int*)(base + yh_b + rate_b + 2 * j_b + perm_b + scr_b + dinv_b + jp_b + gi_b);
  unsigned long long* epoch = (unsigned long long*)((char*)counter + 16);
  int* order = (int*)((char*)counter + 512);
  if (cudaMemsetAsync(counter, 0, 32, st) != cudaSuccess) return UCL_E_CUDA;
  // a batch (no arrival schedule, no live queue) is admitted longest-expected first
  const bool sorted = !arrival_d && q.cap == 0 && nmodels > nslots;
  if (sorted) {
    k_order<<<1, 1024, 0, st>>>(io.params, nmodels, order);
    if (cudaGetLastError() != cudaSuccess) return UCL_E_CUDA;
  }
  const size_t sm = sizeof(T) == 4 ? c->smem32 : c->smem64;
  k_solve_models<T><<<nslots, NT, sm, st>>>(io, A, counter, epoch, arrival_d, sorted ? order : nullptr, q);
  return cuda_status(cudaGetLastError());
}

static int check_solve_args(const ucl_ctx* c, int nmodels, int max_rows, const void* params, const void* phys,
                            const void* abund, const void* nrows, const void* flags, int precision) {
  if (!c || nmodels < 0 || max_rows < 1 || !params || !phys || !abund || !nrows || !flags) return UCL_E_ARG;
  if (precision != UCL_PREC_FP64 && precision != UCL_PREC_MIXED) return UCL_E_ARG;
  return UCL_OK;
}

static int solve_device(ucl_ctx* c, const SolveIO& io, int precision, int max_ctas, void* stream,
                        const double* arrival_d = nullptr) {
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  return precision == UCL_PREC_MIXED ? solve_dev<float>(c, c->ws, io, max_ctas, st, arrival_d)
                                     : solve_dev<double>(c, c->ws, io, max_ctas, st, arrival_d);
}

extern "C" int ucl_solve_models_device(ucl_ctx* c, int nmodels, const ucl_model_params* params_d,
                                       const double* start_d, int max_rows, double* phys_d, double* abund_d,
                                       int* nrows_d, int* flags_d, ucl_model_stats* stats_d, int precision,
                                       int max_ctas, void* stream, double* rates_d) {
  int rc = check_solve_args(c, nmodels, max_rows, params_d, phys_d, abund_d, nrows_d, flags_d, precision);
  if (rc) return rc;
  if (nmodels == 0) return UCL_OK;
  SolveIO io = make_io(c, nmodels, max_rows);
  io.params = params_d; io.start = start_d; io.phys = phys_d; io.abund = abund_d; io.rates = rates_d;
  io.nrows = nrows_d; io.flags = flags_d; io.stats = stats_d;
  return solve_device(c, io, precision, max_ctas, stream);
}

extern "C" int ucl_solve_models_nets_device(ucl_ctx* c, int nmodels, const int* net_of_dev,
                                            const ucl_model_params* params_d, const double* start_d, int max_rows,
                                            double* phys_d, double* abund_d, int* nrows_d, int* flags_d,
                                            ucl_model_stats* stats_d, double* rates_d, int precision, int max_ctas,
                                            void* stream) {
  int rc = check_solve_args(c, nmodels, max_rows, params_d, phys_d, abund_d, nrows_d, flags_d, precision);
  if (rc) return rc;
  if (!net_of_dev) return UCL_E_ARG;
  if (nmodels == 0) return UCL_OK;
  SolveIO io = make_io(c, nmodels, max_rows);
  io.params = params_d; io.start = start_d; io.phys = phys_d; io.abund = abund_d; io.rates = rates_d;
  io.nrows = nrows_d; io.flags = flags_d; io.stats = stats_d; io.net_of = net_of_dev;
  return solve_device(c, io, precision, max_ctas, stream);
}

extern "C" int ucl_solve_models(ucl_ctx* c, int nmodels, const ucl_model_params* params, const double* start,
                                int max_rows, double* phys_out, double* abund_out, int* nrows_out, int* flag_out,
                                ucl_model_stats* stats_out, int precision, double* rates_out) {
  int rc = check_solve_args(c, nmodels, max_rows, params, phys_out, abund_out, nrows_out, flag_out, precision);
  if (rc) return rc;
  if (nmodels == 0) return UCL_OK;
  cudaSetDevice(c->device);
  const int n = c->neq, ns = c->nspec;
  const size_t pb = sizeof(ucl_model_params) * nmodels, sb = start ? (size_t)nmodels * n * 8 : 0,
               phb = (size_t)nmodels * max_rows * UCL_N_PHYS * 8, ab = (size_t)nmodels * max_rows * ns * 8,
               ib = (size_t)nmodels * 4, stb = stats_out ? sizeof(ucl_model_stats) * nmodels : 0,
               rb = rates_out ? (size_t)nmodels * max_rows * c->nreac * 8 : 0;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  rc = c->io.ensure(al(pb) + al(sb) + al(phb) + al(ab) + 2 * al(ib) + al(stb) + al(rb) + 256);
  if (rc) return rc;
  char* b = (char*)c->io.p;
  SolveIO io = make_io(c, nmodels, max_rows);
  io.params = (ucl_model_params*)b;
  b += al(pb);
  io.start = start ? (double*)b : nullptr;
  b += al(sb);
  io.phys = (double*)b;
  b += al(phb);
  io.abund = (double*)b;
  b += al(ab);
  io.nrows = (int*)b;
  b += al(ib);
  io.flags = (int*)b;
  b += al(ib);
  io.stats = stats_out ? (ucl_model_stats*)b : nullptr;
  b += al(stb);
  io.rates = rates_out ? (double*)b : nullptr;
  cudaStream_t s = c->stream;
  if (cudaMemcpyAsync((void*)io.params, params, pb, cudaMemcpyHostToDevice, s) != cudaSuccess) return UCL_E_CUDA;
  if (start && cudaMemcpyAsync((void*)io.start, start, sb, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return UCL_E_CUDA;
  rc = precision == UCL_PREC_MIXED ? solve_dev<float>(c, c->ws, io, 0, s) : solve_dev<double>(c, c->ws, io, 0, s);
  if (rc) return rc;
  if (cudaMemcpyAsync(phys_out, io.phys, phb, cudaMemcpyDeviceToHost, s) != cudaSuccess) return UCL_E_CUDA;
  if (cudaMemcpyAsync(abund_out, io.abund, ab, cudaMemcpyDeviceToHost, s) != cudaSuccess) return UCL_E_CUDA;
  if (cudaMemcpyAsync(nrows_out, io.nrows, ib, cudaMemcpyDeviceToHost, s) != cudaSuccess) return UCL_E_CUDA;
  if (cudaMemcpyAsync(flag_out, io.flags, ib, cudaMemcpyDeviceToHost, s) != cudaSuccess) return UCL_E_CUDA;
  if (stats_out && cudaMemcpyAsync(stats_out, io.stats, stb, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return UCL_E_CUDA;
  if (rates_out && cudaMemcpyAsync(rates_out, io.rates, rb, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return UCL_E_CUDA;
  return cuda_status(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// single-evaluation entry points (parity probes; the context's first network)
extern "C" int ucl_rates_batch(ucl_ctx* c, int nsys, const ucl_model_params* params, double* abund, const double* av,
                               double* phi, double* rates) {
  if (!c || nsys < 0 || !params || !abund || !av || !phi || !rates) return UCL_E_ARG;
  if (nsys == 0) return UCL_OK;
  cudaSetDevice(c->device);
  const DevNet& dn = c->tabs[0].dn;
  const int n = dn.neq, nr = dn.nreac;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t pb = sizeof(ucl_model_params) * nsys, yb = (size_t)nsys * n * 8, vb = (size_t)nsys * 8,
               rb = (size_t)nsys * nr * 8;
  int rc = c->small.ensure(al(pb) + al(yb) + 2 * al(vb) + al(rb));
  if (rc) return rc;
  char* b = (char*)c->small.p;
  ucl_model_params* p_d = (ucl_model_params*)b;
  double* y_d = (double*)(b + al(pb));
  double* av_d = (double*)(b + al(pb) + al(yb));
  double* phi_d = (double*)(b + al(pb) + al(yb) + al(vb));
  double* r_d = (double*)(b + al(pb) + al(yb) + 2 * al(vb));
  cudaStream_t s = c->stream;
  cudaMemcpyAsync(p_d, params, pb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(y_d, abund, yb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(av_d, av, vb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(phi_d, phi, vb, cudaMemcpyHostToDevice, s);
  const size_t sm = (size_t)(n + nr) * 8;
  k_rates<<<nsys, NT, sm, s>>>(dn, p_d, y_d, av_d, phi_d, r_d, nsys);
  if (cudaGetLastError() != cudaSuccess) return UCL_E_CUDA;
  cudaMemcpyAsync(rates, r_d, rb, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(abund, y_d, yb, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(phi, phi_d, vb, cudaMemcpyDeviceToHost, s);
  return cuda_status(cudaStreamSynchronize(s));
}

static int rhs_jac(ucl_ctx* c, int nsys, const ucl_model_params* params, const double* y, const double* rates,
                   const double* av, double* ydot, double* jac) {
  cudaSetDevice(c->device);
  const DevNet& dn = c->tabs[0].dn;
  const int n = dn.neq, nr = dn.nreac;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t pb = sizeof(ucl_model_params) * nsys, yb = (size_t)nsys * n * 8, vb = (size_t)nsys * 8,
               rb = (size_t)nsys * nr * 8, jb = jac ? (size_t)nsys * n * n * 8 : 0,
               jpb = jac ? (size_t)nsys * dn.njch * 8 : 0;
  int rc = c->small.ensure(al(pb) + 2 * al(yb) + al(vb) + al(rb) + al(jb) + al(jpb));
  if (rc) return rc;
  char* b = (char*)c->small.p;
  ucl_model_params* p_d = (ucl_model_params*)b;
  b += al(pb);
  double* y_d = (double*)b;
  b += al(yb);
  double* yd_d = (double*)b;
  b += al(yb);
  double* av_d = (double*)b;
  b += al(vb);
  double* r_d = (double*)b;
  b += al(rb);
  double* j_d = jac ? (double*)b : nullptr;
  b += al(jb);
  double* jp_d = jac ? (double*)b : nullptr;
  cudaStream_t s = c->stream;
  cudaMemcpyAsync(p_d, params, pb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(y_d, y, yb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(av_d, av, vb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(r_d, rates, rb, cudaMemcpyHostToDevice, s);
  const size_t sm = ((size_t)2 * n + 3 * (size_t)nr + (size_t)dn.nchunk + JAC_VEC_DOUBLES) * 8;
  if (cudaFuncSetAttribute(k_rhs_jac, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
    return UCL_E_UNSUPPORTED;
  k_rhs_jac<<<nsys, NT, sm, s>>>(dn, p_d, y_d, r_d, av_d, yd_d, j_d, jp_d, nsys);
  if (cudaGetLastError() != cudaSuccess) return UCL_E_CUDA;
  if (ydot) cudaMemcpyAsync(ydot, yd_d, yb, cudaMemcpyDeviceToHost, s);
  if (jac) cudaMemcpyAsync(jac, j_d, jb, cudaMemcpyDeviceToHost, s);
  return cuda_status(cudaStreamSynchronize(s));
}

extern "C" int ucl_rhs_batch(ucl_ctx* c, int nsys, const ucl_model_params* params, const double* y,
                             const double* rates, const double* av, double* ydot) {
  if (!c || nsys < 0 || !params || !y || !rates || !av || !ydot) return UCL_E_ARG;
  if (nsys == 0) return UCL_OK;
  return rhs_jac(c, nsys, params, y, rates, av, ydot, nullptr);
}

extern "C" int ucl_jac_batch(ucl_ctx* c, int nsys, const ucl_model_params* params, const double* y,
                             const double* rates, const double* av, double* jac) {
  if (!c || nsys < 0 || !params || !y || !rates || !av || !jac) return UCL_E_ARG;
  if (nsys == 0) return UCL_OK;
  return rhs_jac(c, nsys, params, y, rates, av, nullptr, jac);
}

extern "C" int ucl_serve_models_device(ucl_ctx* c, int nmodels, const ucl_model_params* params_d,
                                       const double* arrival_d, const double* start_d, int max_rows, double* phys_d,
                                       double* abund_d, int* nrows_d, int* flags_d, ucl_model_stats* stats_d,
                                       int precision, int max_ctas, void* stream) {
  int rc = check_solve_args(c, nmodels, max_rows, params_d, phys_d, abund_d, nrows_d, flags_d, precision);
  if (rc) return rc;
  if (!arrival_d) return UCL_E_ARG;
  if (nmodels == 0) return UCL_OK;
  SolveIO io = make_io(c, nmodels, max_rows);
  io.params = params_d; io.start = start_d; io.phys = phys_d; io.abund = abund_d;
  io.nrows = nrows_d; io.flags = flags_d; io.stats = stats_d;
  return solve_device(c, io, precision, max_ctas, stream, arrival_d);
}

// ---------------------------------------------------------------------------
// Live serving session: a persistent solver fed through a request ring in
// pinned, device-mapped host memory (LiveQueue in ucl_model.cuh).
struct ucl_server {
  ucl_ctx* c = nullptr;
  int cap = 0, max_rows = 0, precision = 0;
  cudaStream_t kstream = nullptr, cstream = nullptr;
  DevBuf ws, out;
  double *phys = nullptr, *abund = nullptr;
  int *nrows = nullptr, *flags = nullptr;
  ucl_model_stats* stats = nullptr;
  // pinned host memory (and its device aliases)
  ucl_model_params* req_h = nullptr;
  unsigned* ctl_h = nullptr;  // [0] tail, [1] closed, [2..] done[cap]
  int* status_h = nullptr;
  ucl_model_params* req_d = nullptr;
  unsigned* ctl_d = nullptr;
  int* status_d = nullptr;
  std::mutex mu;
  long long next = 0;              // number of the next request
  std::vector<long long> rec_req;  // request held by each record, -1 free
  bool closed = false;
};

static void server_free(ucl_server* s) {
  if (s->kstream) cudaStreamDestroy(s->kstream);
  if (s->cstream) cudaStreamDestroy(s->cstream);
  s->ws.release();
  s->out.release();
  if (s->req_h) cudaFreeHost(s->req_h);
  if (s->ctl_h) cudaFreeHost(s->ctl_h);
  if (s->status_h) cudaFreeHost(s->status_h);
  delete s;
}

extern "C" int ucl_server_open(ucl_ctx* c, int capacity, int max_rows, int precision, int max_ctas,
                               double idle_timeout_s, ucl_server** out) {
  if (!c || !out || capacity < 0 || max_rows < 1 || !(idle_timeout_s >= 0.0)) return UCL_E_ARG;
  if (idle_timeout_s == 0.0) idle_timeout_s = 1200.0;
  if (idle_timeout_s > 80000.0) return UCL_E_ARG;  // the sleep count must fit 32 bits
  if (precision != UCL_PREC_FP64 && precision != UCL_PREC_MIXED) return UCL_E_ARG;
  cudaSetDevice(c->device);
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t rec = al((size_t)max_rows * UCL_N_PHYS * 8) + al((size_t)max_rows * c->nspec * 8);
  const size_t per_rec = rec + 2 * 4 + sizeof(ucl_model_stats);
  if (capacity == 0) {  // as many output records as the context's HBM budget holds
    capacity = (int)std::min<size_t>(1 << 20, c->budget / per_rec);
    if (capacity < 1) return UCL_E_NOMEM;
  }
  ucl_server* s = new ucl_server();
  s->c = c;
  s->cap = capacity;
  s->max_rows = max_rows;
  s->precision = precision;
  s->rec_req.assign(capacity, -1);
  const size_t cap = (size_t)capacity;
  const size_t phb = al(cap * max_rows * UCL_N_PHYS * 8), abb = al(cap * max_rows * c->nspec * 8),
               ib = al(cap * 4), stb = al(cap * sizeof(ucl_model_stats));
  if (s->out.ensure(phb + abb + 2 * ib + stb) != UCL_OK) { server_free(s); return UCL_E_NOMEM; }
  char* b = (char*)s->out.p;
  s->phys = (double*)b;
  s->abund = (double*)(b + phb);
  s->nrows = (int*)(b + phb + abb);
  s->flags = (int*)(b + phb + abb + ib);
  s->stats = (ucl_model_stats*)(b + phb + abb + 2 * ib);
  if (cudaHostAlloc((void**)&s->req_h, cap * sizeof(ucl_model_params), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostAlloc((void**)&s->ctl_h, (cap + 2) * sizeof(unsigned), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostAlloc((void**)&s->status_h, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
    server_free(s);
    return UCL_E_NOMEM;
  }
  memset(s->ctl_h, 0, (cap + 2) * sizeof(unsigned));
  *s->status_h = 0;
  if (cudaHostGetDevicePointer((void**)&s->req_d, s->req_h, 0) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&s->ctl_d, s->ctl_h, 0) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&s->status_d, s->status_h, 0) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->kstream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->cstream, cudaStreamNonBlocking) != cudaSuccess) {
    server_free(s);
    return UCL_E_CUDA;
  }
  SolveIO io = make_io(c, capacity, max_rows);
  io.params = s->req_d;
  io.phys = s->phys; io.abund = s->abund; io.nrows = s->nrows; io.flags = s->flags; io.stats = s->stats;
  LiveQueue q;
  q.req = s->req_d;
  q.tail = s->ctl_d;
  q.closed = s->ctl_d + 1;
  q.done = s->ctl_d + 2;
  q.status = s->status_d;
  q.cap = capacity;
  q.idle_limit = (unsigned)(idle_timeout_s / 20e-6) + 1u;
  const int rc = precision == UCL_PREC_MIXED ? solve_dev<float>(c, s->ws, io, max_ctas, s->kstream, nullptr, q)
                                             : solve_dev<double>(c, s->ws, io, max_ctas, s->kstream, nullptr, q);
  if (rc) { server_free(s); return rc; }
  *out = s;
  return UCL_OK;
}

extern "C" int ucl_server_capacity(const ucl_server* s) { return s ? s->cap : 0; }

extern "C" int ucl_server_submit(ucl_server* s, const ucl_model_params* params, long long* request) {
  if (!s || !params || !request) return UCL_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->closed) return UCL_E_ARG;
  const long long k = s->next;
  const int r = (int)(k % s->cap);
  if (s->rec_req[r] != -1) return UCL_E_AGAIN;  // record still holds an untaken request
  s->req_h[r] = *params;
  s->rec_req[r] = k;
  s->next = k + 1;
  __atomic_store_n(&s->ctl_h[0], (unsigned)(k + 1), __ATOMIC_RELEASE);
  *request = k;
  return UCL_OK;
}

// 1 when request k's outputs are complete, 0 while it is pending
extern "C" int ucl_server_poll(ucl_server* s, long long k) {
  if (!s || k < 0) return UCL_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  const int r = (int)(k % s->cap);
  if (k >= s->next || s->rec_req[r] != k) return UCL_E_ARG;
  if (__atomic_load_n(&s->ctl_h[2 + r], __ATOMIC_ACQUIRE) == (unsigned)(k + 1)) return 1;
  if (__atomic_load_n(s->status_h, __ATOMIC_ACQUIRE) != 0) return UCL_E_TIMEOUT;
  const cudaError_t e = cudaStreamQuery(s->kstream);
  if (e == cudaSuccess) {  // the solver has ended: the request was lost with it
    if (__atomic_load_n(&s->ctl_h[2 + r], __ATOMIC_ACQUIRE) == (unsigned)(k + 1)) return 1;
    return UCL_E_TIMEOUT;
  }
  if (e != cudaErrorNotReady) return UCL_E_CUDA;
  return 0;
}

extern "C" int ucl_server_take(ucl_server* s, long long k, double* phys_out, double* abund_out, int* nrows_out,
                               int* flag_out, ucl_model_stats* stats_out) {
  if (!s || !phys_out || !abund_out || !nrows_out || !flag_out) return UCL_E_ARG;
  const int p = ucl_server_poll(s, k);
  if (p < 0) return p;
  if (p == 0) return UCL_E_AGAIN;
  cudaSetDevice(s->c->device);
  const int r = (int)(k % s->cap), R = s->max_rows, ns = s->c->nspec;
  cudaStream_t st = s->cstream;
  if (cudaMemcpyAsync(phys_out, s->phys + (size_t)r * R * UCL_N_PHYS, (size_t)R * UCL_N_PHYS * 8,
                      cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(abund_out, s->abund + (size_t)r * R * ns, (size_t)R * ns * 8, cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(nrows_out, s->nrows + r, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(flag_out, s->flags + r, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      (stats_out && cudaMemcpyAsync(stats_out, s->stats + r, sizeof(ucl_model_stats), cudaMemcpyDeviceToHost,
                                    st) != cudaSuccess))
    return UCL_E_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return UCL_E_CUDA;
  std::lock_guard<std::mutex> lk(s->mu);
  s->rec_req[r] = -1;
  return UCL_OK;
}

extern "C" int ucl_server_close(ucl_server* s) {
  if (!s) return UCL_E_ARG;
  cudaSetDevice(s->c->device);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->closed = true;
    __atomic_store_n(&s->ctl_h[1], 1u, __ATOMIC_RELEASE);
  }
  const cudaError_t e = cudaStreamSynchronize(s->kstream);
  const int status = *s->status_h;
  server_free(s);
  if (e != cudaSuccess) return UCL_E_CUDA;
  return status ? status : UCL_OK;
}

// batched LU of row-major n x n matrices already on the device
template <typename T>
static int lu_dev(ucl_ctx* c, int nsys, int n, void* mats, int* perm, int* info, cudaStream_t st) {
  const size_t scr_b = (size_t)nsys * 2 * LuCfg<T>::NB * n * sizeof(T);
  int rc = c->small.ensure(scr_b + 256);
  if (rc) return rc;
  const size_t sm = lu_smem_bytes<T>(n);
  if (cudaFuncSetAttribute(k_lu_batch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
    return UCL_E_CUDA;
  k_lu_batch<T><<<nsys, NT, sm, st>>>((T*)mats, n, perm, info, (T*)c->small.p, nsys);
  return cuda_status(cudaGetLastError());
}

extern "C" int ucl_lu_factor_device(ucl_ctx* c, int nsys, int n, int precision, void* mats_dev, int* perm_dev,
                                    int* info_dev, void* stream) {
  if (!c || nsys < 0 || n < 2 || n > MAX_NEQ || (n % 4) != 0 || !mats_dev || !perm_dev || !info_dev)
    return UCL_E_ARG;
  if (precision != UCL_PREC_FP64 && precision != UCL_PREC_MIXED) return UCL_E_ARG;
  if (((uintptr_t)mats_dev & 15) != 0) return UCL_E_ARG;
  if (nsys == 0) return UCL_OK;
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  return precision == UCL_PREC_MIXED ? lu_dev<float>(c, nsys, n, mats_dev, perm_dev, info_dev, st)
                                     : lu_dev<double>(c, nsys, n, mats_dev, perm_dev, info_dev, st);
}

// ---------------------------------------------------------------------------
// Allocation-free batched LU.  The row-interchange scratch lives in a fixed
// file-scope device array; the kernel's grid is capped so that every CTA has
// its own part of it and every CTA is resident at once.  Set-up (symbol
// address, shared-memory attributes, SM count) is done once per device by
// the first call on that device; a set-up that fails is tried again by the
// next call.
static __device__ __align__(256) unsigned char g_lu_scratch[UCL_LU_STATIC_SCRATCH_BYTES];

namespace {
struct StaticLuDev {
  bool ready = false;
  void* scratch = nullptr;
  int nsm = 0;
};
std::mutex g_static_lu_mu;
StaticLuDev g_static_lu[64];
}  // namespace

template <typename T>
static int lu_static(int nsys, int n, void* mats, int* perm, int* info, const StaticLuDev& S, cudaStream_t st) {
  const size_t per = (size_t)2 * LuCfg<T>::NB * n * sizeof(T);
  const int cap = (int)(UCL_LU_STATIC_SCRATCH_BYTES / per);
  if (cap < 1) return UCL_E_ARG;
  const size_t sm = lu_smem_bytes<T>(n);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lu_batch_strided<T>, NT, sm) != cudaSuccess ||
      per_sm < 1)
    return UCL_E_CUDA;
  // no more CTAs than fit on the GPU at once: a CTA beyond that would wait
  // for a second wave while keeping its whole stride of matrices
  const int grid = std::min(std::min(nsys, cap), per_sm * S.nsm);
  k_lu_batch_strided<T><<<grid, NT, sm, st>>>((T*)mats, n, perm, info, (T*)S.scratch, nsys);
  return cuda_status(cudaGetLastError());
}

extern "C" int ucl_lu_factor_device_static(int nsys, int n, int precision, void* mats_dev, int* perm_dev,
                                           int* info_dev, void* stream) {
  if (nsys < 0 || n < 2 || n > MAX_NEQ || (n % 4) != 0 || !mats_dev || !perm_dev || !info_dev) return UCL_E_ARG;
  if (precision != UCL_PREC_FP64 && precision != UCL_PREC_MIXED) return UCL_E_ARG;
  if (((uintptr_t)mats_dev & 15) != 0) return UCL_E_ARG;
  if (nsys == 0) return UCL_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return UCL_E_CUDA;
  StaticLuDev& S = g_static_lu[dev];
  {
    std::lock_guard<std::mutex> lk(g_static_lu_mu);
    if (!S.ready) {
      void* p = nullptr;
      int nsm = 0;
      if (cudaGetSymbolAddress(&p, g_lu_scratch) != cudaSuccess) return UCL_E_CUDA;
      const int sm32 = (int)std::max(lu_smem_bytes<float>(MAX_NEQ), lu_smem_bytes<float>(TC_MAX_N));
      const int sm64 = (int)lu_smem_bytes<double>(MAX_NEQ);
      if (cudaFuncSetAttribute(k_lu_batch_strided<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32) !=
              cudaSuccess ||
          cudaFuncSetAttribute(k_lu_batch_strided<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64) !=
              cudaSuccess ||
          cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
        return UCL_E_CUDA;
      S.scratch = p;
      S.nsm = nsm;
      S.ready = true;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream (there is no context)
  return precision == UCL_PREC_MIXED ? lu_static<float>(nsys, n, mats_dev, perm_dev, info_dev, S, st)
                                     : lu_static<double>(nsys, n, mats_dev, perm_dev, info_dev, S, st);
}

// capacity query used by the host front end
extern "C" int ucl_ctx_slots(const ucl_ctx* c, int precision) {
  if (!c) return 0;
  return precision == UCL_PREC_MIXED ? c->slots_fp32 : c->slots_fp64;
}

extern "C" int ucl_ctx_nspec(const ucl_ctx* c) { return c ? c->nspec : 0; }

extern "C" int ucl_ctx_lu_variant(const ucl_ctx* c, int net, float* us_tensor, float* us_cuda) {
  if (!c || net < 0 || net >= (int)c->tabs.size()) return UCL_E_ARG;
  const DeviceTables& t = c->tabs[net];
  if (us_tensor) *us_tensor = t.lu_us_tc;
  if (us_cuda) *us_cuda = t.lu_us_cuda;
  return t.dn.lu_tc;
}
extern "C" int ucl_ctx_nreac(const ucl_ctx* c) { return c ? c->nreac : 0; }
