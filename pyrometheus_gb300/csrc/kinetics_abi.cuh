// C ABI of a generated mechanism library (declared in
// include/pyrometheus_gb300.h).  Included by the generated translation unit
// after kinetics.cuh.  Every entry point is asynchronous on `stream`,
// allocates nothing, and returns a PyroStatus.
#pragma once

#include "kinetics.cuh"

#ifdef PYRO_UNROLLED
// Straight-line variants (pyro_unrolled::net_rates is generated per
// mechanism): shared memory holds only concentrations and Gibbs energies
// (and the accumulators when PYRO_HOT_COLS is 3); block size HOT_BLOCK.
#define PYRO_HLOOP(i)                                                      \
  for (int64_t i = (int64_t)blockIdx.x * HOT_BLOCK + threadIdx.x; i < n;   \
       i += (int64_t)gridDim.x * HOT_BLOCK)

__device__ __forceinline__ pyro::ColsT<HOT_BLOCK> hcol(double* smem, int q) {
  return pyro::ColsT<HOT_BLOCK>{smem + (size_t)q * NS * HOT_BLOCK +
                                threadIdx.x};
}

__global__ void __launch_bounds__(HOT_BLOCK)
    k_net_production_rates_u(const double* __restrict__ rhop,
                             int64_t rho_inc, const double* __restrict__ Tp,
                             int64_t t_inc, const double* __restrict__ Y,
                             int64_t ldy, double* __restrict__ wdot,
                             int64_t ldw, int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  PYRO_LOG_PRELOAD();
  const auto c = hcol(smem, 0), g = hcol(smem, 1),
             w = hcol(smem, PYRO_HOT_COLS - 1);
  PYRO_HLOOP(i) {
    double wd[NS];
    pyro_unrolled::net_rates(pyro_ld(Tp, t_inc, i), pyro_ld(rhop, rho_inc, i),
                             Y, ldy, i, c, g, w, wd);
#pragma unroll
    for (int k = 0; k < NS; ++k) wdot[(int64_t)k * ldw + i] = wd[k];
  }
}

__global__ void __launch_bounds__(HOT_BLOCK)
    k_fused_step_u(const double* __restrict__ Pp, int64_t p_inc,
                   const double* __restrict__ Tp, int64_t t_inc,
                   const double* __restrict__ Y, int64_t ldy,
                   const double* __restrict__ target, int64_t target_inc,
                   const double* __restrict__ t0, int64_t t0_inc,
                   int do_energy, double tol, int max_iter,
                   double* __restrict__ wdot, int64_t ldw,
                   double* __restrict__ Tout, int* __restrict__ fail_count,
                   int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  PYRO_LOG_PRELOAD();
  const auto c = hcol(smem, 0), g = hcol(smem, 1),
             w = hcol(smem, PYRO_HOT_COLS - 1);
  PYRO_HLOOP(i) {
    const double T = pyro_ld(Tp, t_inc, i);
    double inv_mmw = 0.0;
    for (int k = 0; k < NS; ++k)
      inv_mmw = fma(k_inv_mw[k], __ldg(Y + (int64_t)k * ldy + i), inv_mmw);
    const double rho =
        pyro_ld(Pp, p_inc, i) * (1.0 / inv_mmw) / (GAS_CONSTANT * T);
    double wd[NS];
    pyro_unrolled::net_rates(T, rho, Y, ldy, i, c, g, w, wd);
#pragma unroll
    for (int k = 0; k < NS; ++k) wdot[(int64_t)k * ldw + i] = wd[k];
    double Tn;
    const bool ok = pyro::temperature_newton(
        pyro_ld(target, target_inc, i), pyro_ld(t0, t0_inc, i), Y, ldy, i,
        do_energy != 0, tol, max_iter, Tn);
    Tout[i] = Tn;
    if (!ok && fail_count) atomicAdd(fail_count, 1);
  }
}
#define HOT_COLS PYRO_HOT_COLS
#define K_NET k_net_production_rates_u
#define K_FUSED k_fused_step_u
#else
#define HOT_BLOCK BLOCK
#define HOT_COLS 3
#define K_NET k_net_production_rates
#define K_FUSED k_fused_step
#endif

namespace {

int grid_for(int64_t n) {
  return pyro_grid(n, BLOCK, pyro_sm_count() * BLOCKS_PER_SM);
}

int hot_grid_for(int64_t n) {
  return pyro_grid(n, HOT_BLOCK, pyro_sm_count() * BLOCKS_PER_SM);
}

constexpr size_t smem_cols(int q) { return (size_t)q * NS * BLOCK * 8; }
constexpr size_t hot_smem_cols(int q) {
  return (size_t)q * NS * HOT_BLOCK * 8;
}

// Opt a kernel into more than 48 KB of shared memory (dynamic plus the
// static exp table) when needed.
int prepare_smem(const void* fn, size_t bytes) {
  if (bytes + PYRO_STATIC_SMEM > 48 * 1024) {
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes) != cudaSuccess) {
      (void)cudaGetLastError();
      return PYRO_ERR_LAUNCH;
    }
  }
  return PYRO_OK;
}

}  // namespace

// Threads per block of the straight-line hot kernels (the fused step and
// the net production rates), for callers that size batches in whole waves.
PYRO_EXPORT int pyro_hot_block_size(void) { return HOT_BLOCK; }

PYRO_EXPORT int pyro_mechanism_info(int* n_species, int* n_reactions,
                                    int* n_falloff, int* block_size,
                                    int* table_bytes) {
  if (n_species) *n_species = NS;
  if (n_reactions) *n_reactions = NR;
  if (n_falloff) *n_falloff = NF_REAL;
  if (block_size) *block_size = BLOCK;
  if (table_bytes) *table_bytes = TABLE_BYTES;
  return PYRO_OK;
}

PYRO_EXPORT int pyro_species_property(int which, const double* T,
                                      int64_t t_inc, double* out, int64_t ldo,
                                      int64_t n, cudaStream_t stream) {
  if (n < 0 || which < 0 || which > 6) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!T || !out || ldo < n) return PYRO_ERR_ARGUMENT;
  k_species_prop<<<grid_for(n), BLOCK, 0, stream>>>(which, T, t_inc, out,
                                                    ldo, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_mixture_property(int which, const double* T,
                                      int64_t t_inc, const double* Y,
                                      int64_t ldy, const double* aux,
                                      int64_t aux_inc, double* out, int64_t n,
                                      cudaStream_t stream) {
  if (n < 0 || which < 0 || which > 7) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!Y || !out || ldy < n) return PYRO_ERR_ARGUMENT;
  if (which >= 2 && !T) return PYRO_ERR_ARGUMENT;
  if (which >= 6 && !aux) return PYRO_ERR_ARGUMENT;
  k_mixture_prop<<<grid_for(n), BLOCK, 0, stream>>>(which, T, t_inc, Y, ldy,
                                                    aux, aux_inc, out, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_species_scale(int which, const double* aux,
                                   int64_t aux_inc, const double* Y,
                                   int64_t ldy, double* out, int64_t ldo,
                                   int64_t n, cudaStream_t stream) {
  if (n < 0 || which < 0 || which > 1) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!aux || !Y || !out || ldy < n || ldo < n) return PYRO_ERR_ARGUMENT;
  k_species_scale<<<grid_for(n), BLOCK, 0, stream>>>(which, aux, aux_inc, Y,
                                                     ldy, out, ldo, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_reaction_quantity(int mode, const double* T,
                                       int64_t t_inc, const double* conc,
                                       int64_t ldc, double* out, int64_t ldo,
                                       int64_t n, cudaStream_t stream) {
  if (n < 0 || mode < 0 || mode > 4) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!T || !out || ldo < n) return PYRO_ERR_ARGUMENT;
  if (mode != 0 && (!conc || ldc < n)) return PYRO_ERR_ARGUMENT;
  const size_t sm = smem_cols(2);
  if (prepare_smem((const void*)k_reaction_quantity, sm) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  k_reaction_quantity<<<grid_for(n), BLOCK, sm, stream>>>(mode, T, t_inc,
                                                          conc, ldc, out, ldo,
                                                          n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_net_production_rates(const double* rho, int64_t rho_inc,
                                          const double* T, int64_t t_inc,
                                          const double* Y, int64_t ldy,
                                          double* wdot, int64_t ldw, int64_t n,
                                          cudaStream_t stream) {
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!rho || !T || !Y || !wdot || ldy < n || ldw < n)
    return PYRO_ERR_ARGUMENT;
  const size_t sm = hot_smem_cols(HOT_COLS);
  if (prepare_smem((const void*)K_NET, sm) != PYRO_OK) return PYRO_ERR_LAUNCH;
  K_NET<<<hot_grid_for(n), HOT_BLOCK, sm, stream>>>(rho, rho_inc, T, t_inc, Y,
                                                    ldy, wdot, ldw, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_creation_destruction_rates(
    const double* rho, int64_t rho_inc, const double* T, int64_t t_inc,
    const double* Y, int64_t ldy, double* cdot, double* ddot, int64_t ldo,
    int64_t n, cudaStream_t stream) {
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!rho || !T || !Y || (!cdot && !ddot) || ldy < n || ldo < n)
    return PYRO_ERR_ARGUMENT;
  const size_t sm = smem_cols(4);
  if (prepare_smem((const void*)k_creation_destruction, sm) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  k_creation_destruction<<<grid_for(n), BLOCK, sm, stream>>>(
      rho, rho_inc, T, t_inc, Y, ldy, cdot, ddot, ldo, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_temperature(const double* target, int64_t target_inc,
                                 const double* t0, int64_t t0_inc,
                                 const double* Y, int64_t ldy, int do_energy,
                                 double tol, int max_iter, double* T_out,
                                 int* fail_count, int64_t n,
                                 cudaStream_t stream) {
  if (n < 0 || max_iter < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!target || !t0 || !Y || !T_out || ldy < n) return PYRO_ERR_ARGUMENT;
  k_temperature<<<grid_for(n), BLOCK, 0, stream>>>(
      target, target_inc, t0, t0_inc, Y, ldy, do_energy, tol, max_iter, T_out,
      fail_count, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_fused_step(const double* p, int64_t p_inc,
                                const double* T, int64_t t_inc,
                                const double* Y, int64_t ldy,
                                const double* target, int64_t target_inc,
                                const double* t0, int64_t t0_inc,
                                int do_energy, double tol, int max_iter,
                                double* wdot, int64_t ldw, double* T_out,
                                int* fail_count, int64_t n,
                                cudaStream_t stream) {
  if (n < 0 || max_iter < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!p || !T || !Y || !target || !t0 || !wdot || !T_out || ldy < n ||
      ldw < n)
    return PYRO_ERR_ARGUMENT;
  const size_t sm = hot_smem_cols(HOT_COLS);
  if (prepare_smem((const void*)K_FUSED, sm) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  K_FUSED<<<hot_grid_for(n), HOT_BLOCK, sm, stream>>>(
      p, p_inc, T, t_inc, Y, ldy, target, target_inc, t0, t0_inc, do_energy,
      tol, max_iter, wdot, ldw, T_out, fail_count, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

// ---- reactor source, Jacobian, VJP (csrc/jacobian.cuh) -----------------

PYRO_EXPORT int pyro_reactor_source(const double* p, int64_t p_inc,
                                    const double* T, int64_t t_inc,
                                    const double* Y, int64_t ldy, double* F,
                                    int64_t ldf, int64_t n,
                                    cudaStream_t stream) {
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!p || !T || !Y || !F || ldy < n || ldf < n) return PYRO_ERR_ARGUMENT;
  const size_t sm = smem_cols(3);
  if (prepare_smem((const void*)k_reactor_source, sm) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  k_reactor_source<<<grid_for(n), BLOCK, sm, stream>>>(p, p_inc, T, t_inc, Y,
                                                       ldy, F, ldf, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_reactor_source_dp(const double* p, int64_t p_inc,
                                       const double* T, int64_t t_inc,
                                       const double* Y, int64_t ldy,
                                       double* F, int64_t ldf, int64_t n,
                                       cudaStream_t stream) {
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!p || !T || !Y || !F || ldy < n || ldf < n) return PYRO_ERR_ARGUMENT;
  const size_t sm = (size_t)4 * NS * DPBLOCK * sizeof(double);
  if (prepare_smem((const void*)k_reactor_source_dp, sm) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  k_reactor_source_dp<<<pyro_grid(n, DPBLOCK, pyro_sm_count() * 16),
                        DPBLOCK, sm, stream>>>(p, p_inc, T, t_inc, Y, ldy, F,
                                               ldf, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

namespace {
int launch_reactor_jacobian(const double* p, int64_t p_inc, const double* T,
                            int64_t t_inc, const double* Y, int64_t ldy,
                            double* F, int64_t ldf, double* J, int64_t ldj,
                            int64_t n, cudaStream_t stream) {
  const size_t sm = (size_t)JGROUPS * JW_DOUBLES * sizeof(double);
  if (prepare_smem((const void*)k_reactor_jacobian, sm) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  const int64_t blocks = (n + JGROUPS - 1) / JGROUPS;
  const int grid =
      (int)(blocks < (int64_t)pyro_sm_count() * 8 ? blocks
                                                   : (int64_t)pyro_sm_count() * 8);
  k_reactor_jacobian<<<grid, JGROUPS * JGROUP, sm, stream>>>(
      p, p_inc, T, t_inc, Y, ldy, J, ldj, F, ldf, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
}  // namespace

PYRO_EXPORT int pyro_reactor_jacobian(const double* p, int64_t p_inc,
                                      const double* T, int64_t t_inc,
                                      const double* Y, int64_t ldy, double* J,
                                      int64_t ldj, int64_t n,
                                      cudaStream_t stream) {
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!p || !T || !Y || !J || ldy < n ||
      ldj < (int64_t)(NS + 1) * (NS + 1))
    return PYRO_ERR_ARGUMENT;
  return launch_reactor_jacobian(p, p_inc, T, t_inc, Y, ldy, nullptr, 0, J,
                                 ldj, n, stream);
}

PYRO_EXPORT int pyro_reactor_source_jacobian(
    const double* p, int64_t p_inc, const double* T, int64_t t_inc,
    const double* Y, int64_t ldy, double* F, int64_t ldf, double* J,
    int64_t ldj, int64_t n, cudaStream_t stream) {
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!p || !T || !Y || !F || !J || ldy < n || ldf < n ||
      ldj < (int64_t)(NS + 1) * (NS + 1))
    return PYRO_ERR_ARGUMENT;
  return launch_reactor_jacobian(p, p_inc, T, t_inc, Y, ldy, F, ldf, J, ldj,
                                 n, stream);
}

PYRO_EXPORT int pyro_reactor_vjp(const double* p, int64_t p_inc,
                                 const double* T, int64_t t_inc,
                                 const double* Y, int64_t ldy,
                                 const double* V, int64_t ldv, double* gT,
                                 double* gY, int64_t ldg, double* gp,
                                 int64_t n, cudaStream_t stream) {
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!p || !T || !Y || !V || !gT || !gY || ldy < n || ldv < n || ldg < n)
    return PYRO_ERR_ARGUMENT;
  const size_t sm = (size_t)5 * NS * VBLOCK * sizeof(double);
  if (prepare_smem((const void*)k_reactor_vjp, sm) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  k_reactor_vjp<<<pyro_grid(n, VBLOCK, pyro_sm_count() * 16), VBLOCK, sm,
                  stream>>>(p, p_inc, T, t_inc, Y, ldy, V, ldv, gT, gY, ldg,
                            gp, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
