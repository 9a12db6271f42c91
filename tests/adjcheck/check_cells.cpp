// Finite-difference check of the generated per-cell reverse sweeps
// (csrc/adj_cells.cuh) in double precision on the host: for random inputs
// and output weights w, the adjoint's input gradient of <w, f(x)> must match
// central differences.  Prints one line per cell: name, max relative error.
// TEST INFRASTRUCTURE (built and run by tests/test_adjoint_cells.py).
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#define __host__
#define __device__
#define __forceinline__ inline
#include "../../g3m3_gb300/csrc/adj_cells.cuh"

using namespace g3m3::adj;

template <class C>
double check(const char* name, std::mt19937_64& rng, const std::vector<double>& par, double lo, double hi,
             int trials) {
  std::uniform_real_distribution<double> U(lo, hi), W(-1.0, 1.0);
  double worst = 0.0;
  for (int t = 0; t < trials; t++) {
    std::vector<double> x(C::NIN), w(C::NOUT), g(C::NIN, 0.0), y(C::NOUT);
    for (auto& v : x) v = U(rng);
    for (auto& v : w) v = W(rng);
    C::adj(x.data(), par.data(), w.data(), [&](int s, double v) { g[s] += v; });
    for (int i = 0; i < C::NIN; i++) {
      const double h = 1e-6 * std::fmax(1.0, std::fabs(x[i]));
      std::vector<double> xp = x, xm = x;
      xp[i] += h;
      xm[i] -= h;
      double fp = 0.0, fm = 0.0;
      C::fwd(xp.data(), par.data(), y.data());
      for (int o = 0; o < C::NOUT; o++) fp += w[o] * y[o];
      C::fwd(xm.data(), par.data(), y.data());
      for (int o = 0; o < C::NOUT; o++) fm += w[o] * y[o];
      const double fd = (fp - fm) / (2.0 * h);
      const double err = std::fabs(fd - g[i]) / std::fmax(1e-6, std::fmax(std::fabs(fd), std::fabs(g[i])));
      if (err > worst) worst = err;
    }
  }
  std::printf("%s %.3e\n", name, worst);
  return worst;
}

int main() {
  std::mt19937_64 rng(20261204);
  // push_ion: rho and pressures positive, B of order 1; bmax small enough that both skin branches occur
  check<push_ion_cell<double>>("push_ion_cell", rng,
                               {0.01, 1.0, 1.0, 1.0, 1.0, 0.7, 0.9, 0.3, 1.0e-3, 4.0, 2.0, 1.2, -0.8, 0.5}, 0.5, 1.5,
                               20);
  check<push_ion_cell<double>>("push_ion_cell_strongB", rng,
                               {0.01, 1.0, 1.0, 1.0, 1.0, 0.7, 0.2, 0.3, 1.0e-3, 4.0, 2.0, 1.2, -0.8, 0.5}, 0.5, 1.5,
                               20);
  check<push_elec_cell<double>>("push_elec_cell", rng, {0.01, 1.6667, 0.6667, 1.0, 1.0, 1.0}, -1.0, 1.0, 20);
  check<push_bfld_cell<double>>("push_bfld_cell", rng, {0.01, 1.0, 1.0, 1.0}, -1.0, 1.0, 20);
  check<curl_cell<double>>("curl_cell", rng, {1.0, 1.0, 1.0}, -1.0, 1.0, 20);
  check<total_b_cell<double>>("total_b_cell", rng, {0.3, -0.2, 0.5, 1.0e-5}, -1.0, 1.0, 20);
  check<evel_cell<double>>("evel_cell", rng, {1.0, 1.0, 16.0, 0.9}, 0.5, 1.5, 20);
  check<vtot_cell<double>>("vtot_cell", rng, {}, 0.5, 1.5, 20);
  check<bande_cell<double>>("bande_cell", rng, {1.0, 1.0, 16.0, 0.9, 1.0, 1.0, 1.0, 0.3}, 0.5, 1.5, 20);
  check<lap_speed_cell<double>>("lap_speed_cell", rng, {1.0e-5}, 0.2, 1.5, 20);
  check<lap_jump_cell<double>>("lap_jump_cell", rng, {}, -1.0, 1.0, 20);
  check<lap_field_cell<double>>("lap_field_cell", rng, {0.1, 0.01}, -1.0, 1.0, 20);
  check<fcs_flux_cell<double>>("fcs_flux_cell", rng, {0.05}, -1.0, 1.0, 200);
  return 0;
}
