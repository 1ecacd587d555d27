// C entry points around the reference's gridless relativistic Boris mover
// (srcEarth/gridless/GridlessParticleMovers.cpp:781 BorisStep) and its dipole
// (srcEarth/gridless/DipoleInterface.h:99 GetB_Tesla), compiled from the
// reference tree into oracle/_ref/gridless_ref.so.
//
// Test infrastructure: used to pin the oracle's tracer and to generate the
// golden trajectories committed under tests/golden/.  The step-size rule is
// the gyro-angle limiter of CutoffRigidityGridless.cpp:1190-1197.
#include <cmath>

#include "DipoleInterface.h"
#include "GridlessParticleMovers.h"

namespace Earth {
namespace GridlessMode {
namespace Dipole {
Params gParams;
}
}  // namespace GridlessMode
}  // namespace Earth

namespace {
struct DipolePlusUniform : public IGridlessFieldEvaluator {
  double scale = 1.0;
  double ext[3] = {0, 0, 0};
  void GetB_T(const V3& x, V3& B) const override {
    double xm[3] = {x.x, x.y, x.z}, b[3];
    Earth::GridlessMode::Dipole::GetB_Tesla(xm, b);
    B = V3{scale * b[0] + ext[0], scale * b[1] + ext[1], scale * b[2] + ext[2]};
  }
};
}  // namespace

extern "C" {

// Equatorial surface field of the reference dipole (DipoleInterface.h:70).
double gridless_ref_beq() { return Earth::GridlessMode::Dipole::B_eq_Re; }
double gridless_ref_re() { return Earth::GridlessMode::Dipole::Re_m; }

// Trace n particles; status 1 = r < r_in, 2 = r > r_out, 0 = step cap.
long gridless_ref_trace(long n, double* x, double* p, int* status, long* steps, double q,
                        double m0, double b_eq, const double* b_ext, double r_in, double r_out,
                        long max_steps, double dphi_max, double dt_max) {
  DipolePlusUniform f;
  f.scale = b_eq / Earth::GridlessMode::Dipole::B_eq_Re;
  for (int d = 0; d < 3; d++) f.ext[d] = b_ext[d];
  long total = 0;
  for (long i = 0; i < n; i++) {
    V3 xx{x[3 * i], x[3 * i + 1], x[3 * i + 2]}, pp{p[3 * i], p[3 * i + 1], p[3 * i + 2]};
    long s = 0;
    int st = 0;
    while (s < max_steps) {
      V3 B;
      f.GetB_T(xx, B);
      double Bm = std::sqrt(B.x * B.x + B.y * B.y + B.z * B.z);
      double mc = m0 * 299792458.0;
      double gam = std::sqrt(1.0 + (pp.x * pp.x + pp.y * pp.y + pp.z * pp.z) / (mc * mc));
      double dt = dt_max;
      if (Bm > 0.0) {
        double om = std::fabs(q) * Bm / (gam * m0);
        if (om > 0.0) dt = std::min(dt, dphi_max / om);
      }
      BorisStep(xx, pp, q, m0, dt, f);
      s++;
      double r = std::sqrt(xx.x * xx.x + xx.y * xx.y + xx.z * xx.z);
      if (r < r_in) { st = 1; break; }
      if (r > r_out) { st = 2; break; }
    }
    x[3 * i] = xx.x; x[3 * i + 1] = xx.y; x[3 * i + 2] = xx.z;
    p[3 * i] = pp.x; p[3 * i + 1] = pp.y; p[3 * i + 2] = pp.z;
    status[i] = st;
    steps[i] = s;
    total += s;
  }
  return total;
}
}
