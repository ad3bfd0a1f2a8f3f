// Hot-core physics on the device: the physics module of hotcore.f90,
// selected per model by ucl_model_params::hotcore (the temp_indx 1-6 of
// uclchem.model.hot_core: protostar masses 1, 5, 10, 15, 25, 60 Msun).  The
// gas and dust temperature of the parcel follow the ramp
//   T = initialTemp + a_m * t^b_m * (r/rout)^-1/2,  capped at maxTemperature
// (hotcore.f90:70-79, t in years, r the parcel's depth: rout for one
// parcel), updated after each interval, and the output times follow the
// module's own schedule (:50-66).  On a three-phase network (the default
// one) the module's sublimation routine does nothing (:82-96): the
// thermal desorption of the ices is in the chemistry.
#pragma once
#include "ucl_chem.cuh"

namespace ucl {

// hotcore.f90:13-14: tempa are 'd' literals, tempb default-REAL ones
__device__ __forceinline__ double hc_tempa(int m) {
  switch (m) {
    case 1: return 1.927e-1;
    case 2: return 4.8560e-2;
    case 3: return 7.8470e-3;
    case 4: return 9.6966e-4;
    case 5: return 1.706e-4;
    default: return 4.74e-7;
  }
}
__device__ __forceinline__ double hc_tempb(int m) {
  switch (m) {
    case 1: return (double)0.5339f;
    case 2: return (double)0.6255f;
    case 3: return (double)0.8395f;
    case 4: return (double)1.085f;
    case 5: return (double)1.289f;
    default: return (double)1.98f;
  }
}

// updateTargetTime of the hot-core module (hotcore.f90:50-66), seconds
__device__ __forceinline__ double hc_target_time(double ty, double spy) {
  if (ty > 1.0e6) return (ty + 1.0e5) * spy;
  if (ty > 1.0e5) return (ty + 1.0e4) * spy;
  if (ty > 1.0e4) return (ty + 1000.0) * spy;
  if (ty > 1000) return (ty + 100.0) * spy;
  if (ty > 100) return (ty + 10.0) * spy;
  if (ty > 0.0) return (ty * 10.0) * spy;
  return spy * 1.0e-7;
}

// updatePhysics of the hot-core module (hotcore.f90:70-79) for one parcel:
// the new gas temperature from the old one, at time t (s)
__device__ __noinline__ double hc_temperature(int m, double T, double t, double initialTemp, double maxTemp,
                                             double cloudSize, double rout, int points) {
  if (!(T < maxTemp)) return T;
  double g = (cloudSize / (rout * cK.PC)) * (double)((float)1 / (float)points);
  g = pow(g, -0.5);
  T = initialTemp + ((hc_tempa(m) * pow(t / cK.SECONDS_PER_YEAR, hc_tempb(m))) * g);
  if (T > maxTemp) T = maxTemp;
  return T;
}

}  // namespace ucl
