// TEST INFRASTRUCTURE / CPU BASELINE ONLY: a batch driver around the C++20
// header that the reference's own C++ target (pyrometheus/codegen/cpp.py)
// generates for a mechanism.  The header is rendered by oracle/ref_cpp.py
// into oracle/_ref/ and never committed; this file only loops over states
// and calls the header's per-state functions (get_density,
// get_net_production_rates, get_temperature), so the timed CPU path is the
// reference's own generated code.  Build: see oracle/ref_cpp.py.
#include <cstdint>

#include REF_HEADER

#ifdef _OPENMP
#include <omp.h>
#endif

using Thermo = pyro::Thermochemistry<double>;
using SpeciesT = Thermo::SpeciesT;

extern "C" {

int ref_num_species() { return Thermo::num_species; }

int ref_num_reactions() { return Thermo::num_reactions; }

// One pass per state of density, net production rates and the temperature
// Newton from the internal energy (the headline workload): p, T, e [n];
// Y [S][ldy]; wdot [S][ldw]; T_out [n]; nthreads OpenMP threads.
int ref_fused_step(int64_t n, const double* p, const double* T,
                   const double* Y, int64_t ldy, const double* e, double t0,
                   double* wdot, int64_t ldw, double* T_out, int nthreads) {
  if (n < 0 || ldy < n || ldw < n || nthreads < 1) return 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    SpeciesT y;
    for (int k = 0; k < Thermo::num_species; ++k) y[k] = Y[k * ldy + i];
    const double rho = Thermo::get_density(p[i], T[i], y);
    const SpeciesT w = Thermo::get_net_production_rates(rho, T[i], y);
    for (int k = 0; k < Thermo::num_species; ++k) wdot[k * ldw + i] = w[k];
    T_out[i] = Thermo::get_temperature(e[i], t0, y, true);
  }
  return 0;
}

}  // extern "C"
