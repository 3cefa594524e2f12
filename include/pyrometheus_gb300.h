/*
 * pyrometheus_gb300 C ABI.
 *
 * A mechanism library (libpyro_<mechanism>_<hash>.so) is generated by the
 * `cuda` code-generation target and exports the entry points below, one
 * per method of the reference's generated Thermochemistry class
 * (pyrometheus/codegen/python.py).  Every entry point:
 *
 *   - takes caller-owned device pointers, sizes and strides in elements,
 *     and a cudaStream_t; it is asynchronous on that stream;
 *   - allocates nothing;
 *   - returns a PyroStatus (0 ok, 1 bad argument, 2 launch failure,
 *     3 non-convergence, 4 unsupported option).
 *
 * Layouts (FP64): per-species and per-reaction arrays are species-major,
 * x[k * ld + i] for state i (ld >= n).  A per-state scalar argument is a
 * pointer plus an increment: inc = 1 for an array of n values, inc = 0 to
 * broadcast one device value to every state (the reference's scalar
 * arguments).
 */
#ifndef PYROMETHEUS_GB300_H
#define PYROMETHEUS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* cudaStream_t;

enum PyroStatus {
  PYRO_OK = 0,
  PYRO_ERR_ARGUMENT = 1,
  PYRO_ERR_LAUNCH = 2,
  PYRO_ERR_NOT_CONVERGED = 3,
  PYRO_ERR_UNSUPPORTED = 4
};

/* ---- mechanism library (generated per mechanism) ------------------------ */

/* Sizes of the compiled mechanism (num_species, num_reactions, num_falloff:
 * python.py:180-185), the kernels' block size and table footprint. */
int pyro_mechanism_info(int* n_species, int* n_reactions, int* n_falloff,
                        int* block_size, int* table_bytes);

/* Threads per block of the hot kernels (pyro_fused_step,
 * pyro_net_production_rates): one block per SM runs at a time, so batches
 * of a multiple of (SM count x this) states fill whole waves. */
int pyro_hot_block_size(void);

/* Species NASA-7 properties at T, out[S][ldo]; which:
 *   0 cp/R          get_species_specific_heats_r            python.py:334
 *   1 h/RT          get_species_enthalpies_rt               python.py:341
 *   2 s/R           get_species_entropies_r                 python.py:348
 *   3 g/RT          get_species_gibbs_rt                    python.py:355
 *   4 d(cp/R)/dT    get_species_specific_heats_r_derivative python.py:313
 *   5 d(h/RT)/dT    get_species_enthalpies_rt_derivative    python.py:320
 *   6 d(s/R)/dT     get_species_entropies_rt_derivative     python.py:327 */
int pyro_species_property(int which, const double* T, int64_t t_inc,
                          double* out, int64_t ldo, int64_t n,
                          cudaStream_t stream);

/* Mixture properties, out[n]; which:
 *   0 mixture molecular weight   get_mixture_molecular_weight  python.py:265
 *   1 specific gas constant      get_specific_gas_constant     python.py:248
 *   2 cp (mass)                  get_mixture_specific_heat_cp_mass :293
 *   3 cv (mass)                  get_mixture_specific_heat_cv_mass :298
 *   4 h (mass)                   get_mixture_enthalpy_mass         :303
 *   5 e (mass)                   get_mixture_internal_energy_mass  :308
 *   6 density, aux = pressure    get_density                   python.py:255
 *   7 pressure, aux = density    get_pressure                  python.py:260
 * T may be NULL for which 0-1, aux must be given for which 6-7. */
int pyro_mixture_property(int which, const double* T, int64_t t_inc,
                          const double* Y, int64_t ldy, const double* aux,
                          int64_t aux_inc, double* out, int64_t n,
                          cudaStream_t stream);

/* out[S][ldo]; which 0: concentrations, aux = rho
 * (get_concentrations, python.py:272); which 1: mole fractions, aux =
 * mixture molecular weight (get_mole_fractions, python.py:279). */
int pyro_species_scale(int which, const double* aux, int64_t aux_inc,
                       const double* Y, int64_t ldy, double* out, int64_t ldo,
                       int64_t n, cudaStream_t stream);

/* Per-reaction quantities from T and concentrations, out[R][ldo]; mode:
 *   0 log equilibrium constants  get_equilibrium_constants  python.py:360
 *     (conc may be NULL)
 *   1 forward rate coefficients  get_fwd_rate_coefficients  python.py:453
 *     (falloff slots as get_falloff_rates writes them, python.py:399)
 *   2 net rates of progress      get_net_rates_of_progress  python.py:475
 *   3 forward rates of progress  get_fwd_rates_of_progress  python.py:497
 *   4 reverse rates of progress  get_rev_rates_of_progress  python.py:506 */
int pyro_reaction_quantity(int mode, const double* T, int64_t t_inc,
                           const double* conc, int64_t ldc, double* out,
                           int64_t ldo, int64_t n, cudaStream_t stream);

/* Net molar production rates wdot[S][ldw] from (rho, T, Y):
 * get_net_production_rates, python.py:486.  The hot path. */
int pyro_net_production_rates(const double* rho, int64_t rho_inc,
                              const double* T, int64_t t_inc,
                              const double* Y, int64_t ldy, double* wdot,
                              int64_t ldw, int64_t n, cudaStream_t stream);

/* Creation and destruction rates (either output may be NULL):
 * get_creation_destruction_rates, python.py:543 (and get_creation_rates
 * :517, get_destruction_rates :530). */
int pyro_creation_destruction_rates(const double* rho, int64_t rho_inc,
                                    const double* T, int64_t t_inc,
                                    const double* Y, int64_t ldy,
                                    double* cdot, double* ddot, int64_t ldo,
                                    int64_t n, cudaStream_t stream);

/* Temperature from mass-specific internal energy (do_energy != 0) or
 * enthalpy: get_temperature, python.py:375 (tol 1e-6, max_iter 500 there).
 * Per-state Newton; states that do not reach |dT| < tol within max_iter are
 * counted into *fail_count (device int, may be NULL; the caller zeroes it).
 * The caller raises the reference's RuntimeError when it is non-zero. */
int pyro_temperature(const double* target, int64_t target_inc,
                     const double* t0, int64_t t0_inc, const double* Y,
                     int64_t ldy, int do_energy, double tol, int max_iter,
                     double* T_out, int* fail_count, int64_t n,
                     cudaStream_t stream);

/* One pass per state of get_density(p, T, Y) -> get_net_production_rates
 * -> get_temperature(target, t0, Y, do_energy): the chain of the 0-D
 * reactor right-hand side (examples/free_flame/reactors.py:115-123) and the
 * flamelet source terms (flamelets/equations.py:313-359). */
int pyro_fused_step(const double* p, int64_t p_inc, const double* T,
                    int64_t t_inc, const double* Y, int64_t ldy,
                    const double* target, int64_t target_inc,
                    const double* t0, int64_t t0_inc, int do_energy,
                    double tol, int max_iter, double* wdot, int64_t ldw,
                    double* T_out, int* fail_count, int64_t n,
                    cudaStream_t stream);

/* Reactor right-hand side f = (dT/dt, dY_1/dt .. dY_S/dt) of the adiabatic
 * constant-pressure 0-D reactor, [S+1][ldf]: the function the reference's
 * reactors integrate and differentiate (examples/free_flame/reactors.py:
 * 115-125; flamelets/equations.py:124-129 for the Jacobian). */
int pyro_reactor_source(const double* p, int64_t p_inc, const double* T,
                        int64_t t_inc, const double* Y, int64_t ldy,
                        double* F, int64_t ldf, int64_t n,
                        cudaStream_t stream);

/* Its Jacobian d f / d (T, Y) per state, J[n][ldj] with the (S+1) x (S+1)
 * block row-major at J + i * ldj (ldj >= (S+1)^2): replaces
 * jax.jacfwd(rhs) of reactors.py:125 / equations.py:124-129. */
int pyro_reactor_jacobian(const double* p, int64_t p_inc, const double* T,
                          int64_t t_inc, const double* Y, int64_t ldy,
                          double* J, int64_t ldj, int64_t n,
                          cudaStream_t stream);

/* The source and its Jacobian in one pass: F[S+1][ldf] as
 * pyro_reactor_source and J as pyro_reactor_jacobian, from the rates the
 * Jacobian kernel forms anyway.  Replaces the primal-and-tangent pair that
 * jax.jacfwd(rhs) yields in one trace (examples/free_flame/reactors.py:
 * 115-125, flamelets/equations.py:124-129) -- and the two separate calls
 * a caller of the generated class would otherwise make. */
int pyro_reactor_source_jacobian(const double* p, int64_t p_inc,
                                 const double* T, int64_t t_inc,
                                 const double* Y, int64_t ldy, double* F,
                                 int64_t ldf, double* J, int64_t ldj,
                                 int64_t n, cudaStream_t stream);

/* Vector-Jacobian product v^T df/d(T, Y) and v^T df/dp for cotangents
 * V[S+1][ldv]: gT[n], gY[S][ldg], gp[n] (gp may be NULL); the reverse-mode
 * counterpart of jax.vjp over the same function. */
int pyro_reactor_vjp(const double* p, int64_t p_inc, const double* T,
                     int64_t t_inc, const double* Y, int64_t ldy,
                     const double* V, int64_t ldv, double* gT, double* gY,
                     int64_t ldg, double* gp, int64_t n, cudaStream_t stream);

/* Integrate cells [0, n) of a reactor pool with the fused per-cell
 * variable-step BDF2 / chord-Newton kernel, up to `attempts` step attempts
 * per cell in this call (the reference steps one reactor at a time with
 * Crank-Nicolson and a Newton loop around jnp.linalg.solve,
 * examples/free_flame/time_integ.py:70-106).  Per cell (leading dimension
 * ld >= n): y, y_prev, f_n [S+1][ld]; p, t, t_end, h, h_prev, g_lu, crate
 * [ld] doubles; nsteps, nattempts, jage [ld] int64; active, failed, jstale,
 * done [ld] bytes; J, M [(S+1)^2][ld] doubles; piv [S+1][ld] ints.  Cells
 * with active == 0 are skipped; a cell that reaches t_end or fails gets
 * active = 0 and done = 1 (failed = 1 on failure).  With slots != NULL the
 * call integrates the n cells slots[0..n) instead (the active cells of a
 * fragmented pool, so no thread idles on a finished cell).  Allocates
 * nothing. */
int pyro_reactor_bdf2(double* y, double* y_prev, double* f_n, int64_t ld,
                      const double* p, double* t, const double* t_end,
                      double* h, double* h_prev, double* g_lu, double* crate,
                      int64_t* nsteps, int64_t* nattempts, int64_t* jage,
                      unsigned char* active, unsigned char* failed,
                      unsigned char* jstale, unsigned char* done, double* J,
                      double* M, int* piv, const int64_t* slots, int64_t n,
                      int attempts, double rtol, double atol,
                      int64_t max_attempts, cudaStream_t stream);

/* Steady-flamelet residual, R[nv][ldr] = chi/2 Lap(phi) + S(phi) m - BC,
 * for flamelets packed along rows (system s owns rows [row_off[s],
 * row_off[s+1]), at least 3; sys_of_row[rows] gives s; uniform grid with
 * inv_dx2[s] = 1/dx^2): FlameletEquations.rhs,
 * pyrometheus/flamelets/equations.py:167-227, with the Laplacian of
 * onedim_laplacian.py:182-212 and source_terms equations.py:313-359.
 * Inputs: T[rows] (from get_temperature_from_enthalpy), h[rows],
 * Y[S][ldy], F[S+1][ldf] the reactor source at (p, T, Y) (rows 1.. are
 * W_k w_k / rho), chi and visc [rows], h_ox/h_fu [nsys], y_ox/y_fu
 * [S][ldb] (ldb >= nsys). */
int pyro_flamelet_residual(const double* p, int64_t p_inc, const double* T,
                           const double* h, const double* Y, int64_t ldy,
                           const double* F, int64_t ldf, const double* chi,
                           const double* visc, const int64_t* row_off,
                           const int* sys_of_row, const double* inv_dx2,
                           const double* h_ox, const double* h_fu,
                           const double* y_ox, const double* y_fu,
                           int64_t ldb, double* R, int64_t ldr, int64_t rows,
                           cudaStream_t stream);

/* Block-tridiagonal Jacobian of that residual w.r.t. (h, Y):
 * FlameletEquations.jac, equations.py:228-282, and
 * Laplacian.assemble_block_form, onedim_laplacian.py:144-180.  On entry
 * C[rows][nv][nv] holds pyro_reactor_jacobian at (p, T, Y); it is turned in
 * place into the central blocks (chain rule through T(h, Y), viscous
 * enthalpy row, zero source blocks at the boundary points, chi/2 times the
 * Laplacian diagonal); L and U receive the packed sub/super-diagonal blocks
 * pyro_block_thomas takes (the last row of each flamelet zero). */
int pyro_flamelet_blocks(const double* p, int64_t p_inc, const double* T,
                         const double* Y, int64_t ldy, const double* chi,
                         const double* visc, const int64_t* row_off,
                         const int* sys_of_row, const double* inv_dx2,
                         double* L, double* C, double* U, int64_t rows,
                         cudaStream_t stream);

/* Matrix-free Jacobian action A v = chi/2 Lap(v) + dS/dphi v per point,
 * A[S+1][lda] for directions V[S+1][ldv]: FlameletEquations.jacobian_action,
 * pyrometheus/flamelets/equations.py:411-450.  Every point keeps its source
 * Jacobian (the boundary points included, unlike the blocks) and the
 * Laplacian's boundary rows are v / dx^2.  J[rows][nv][nv] holds
 * pyro_reactor_jacobian at (p, T, Y) (read only); other arguments as for
 * pyro_flamelet_blocks. */
int pyro_flamelet_jacobian_action(const double* p, int64_t p_inc,
                                  const double* T, const double* Y,
                                  int64_t ldy, const double* J,
                                  const double* V, int64_t ldv,
                                  const double* chi, const double* visc,
                                  const int64_t* row_off,
                                  const int* sys_of_row,
                                  const double* inv_dx2, double* A,
                                  int64_t lda, int64_t rows,
                                  cudaStream_t stream);

/* dF/dp [S+1][ldf] of the reactor source at fixed (T, Y), in forward mode
 * (the concentrations and [M] scale with p): the pressure derivative the
 * reference takes with jacfwd, FlameletEquations.source_gradient_wrt_pressure,
 * pyrometheus/flamelets/equations.py:130-134. */
int pyro_reactor_source_dp(const double* p, int64_t p_inc, const double* T,
                           int64_t t_inc, const double* Y, int64_t ldy,
                           double* F, int64_t ldf, int64_t n,
                           cudaStream_t stream);

/* Adjoint operator of the compressible-EOS consistency solves,
 * FlameletEquations.adjoint_operator, equations.py:451-516 (used by
 * CompressibleEOS.enthalpy_gradient / eos_gradient,
 * thermodynamic_consistency.py:105-307).  Same arguments and in-place use
 * of C as pyro_flamelet_blocks; the result: interior C_i = Lap_c I +
 * (2 / chi_i) (dS/dphi_i)^T, boundary C_i = chi_i / 2 dx^-2 I, L and U the
 * Laplacian's couplings dx^-2 I without the chi / 2 factor. */
int pyro_flamelet_adjoint_blocks(const double* p, int64_t p_inc,
                                 const double* T, const double* Y,
                                 int64_t ldy, const double* chi,
                                 const double* visc, const int64_t* row_off,
                                 const int* sys_of_row,
                                 const double* inv_dx2, double* L, double* C,
                                 double* U, int64_t rows,
                                 cudaStream_t stream);

/* rt[rows] = R_u T / W_mix and, when J is not NULL, its gradient with
 * respect to (h, Y) at T(h, Y), J[S+1][ldj]: compressible_eos_rt and
 * compressible_eos_rt_jacobian, equations.py:136-147,517-535. */
int pyro_flamelet_eos_rt(const double* T, const double* Y, int64_t ldy,
                         double* rt, double* J, int64_t ldj, int64_t rows,
                         cudaStream_t stream);

/* ---- mixture-averaged transport (python.py:564-641) ---------------------
 * Present in every mechanism library; for a mechanism generated without
 * transport fits the three compute entry points return
 * PYRO_ERR_UNSUPPORTED. */

/* available = 1 when the library carries transport fits; symmetric = 1
 * when the binary-diffusivity fits satisfy D_ij = D_ji. */
int pyro_transport_info(int* available, int* symmetric);

/* Species transport at T, out[S][ldo]; which:
 *   0 viscosities            get_species_viscosities            python.py:564
 *   1 thermal conductivities get_species_thermal_conductivities python.py:573 */
int pyro_species_transport(int which, const double* T, int64_t t_inc,
                           double* out, int64_t ldo, int64_t n,
                           cudaStream_t stream);

/* Binary diffusivities D_ij at T, out[(i S + j) ldo + state]:
 * get_species_binary_mass_diffusivities, python.py:582-593. */
int pyro_binary_diffusivities(const double* T, int64_t t_inc, double* out,
                              int64_t ldo, int64_t n, cudaStream_t stream);

/* Mixture-averaged viscosity mu[n] (get_mixture_viscosity_mixavg,
 * python.py:595-605), thermal conductivity lam[n]
 * (get_mixture_thermal_conductivity_mixavg, python.py:607-613) and species
 * diffusivities D[S][ldd] (get_species_mass_diffusivities_mixavg,
 * python.py:615-641) in one pass; a NULL output is skipped, and P may be
 * NULL when D is. */
int pyro_transport_mixavg(const double* P, int64_t p_inc, const double* T,
                          int64_t t_inc, const double* Y, int64_t ldy,
                          double* mu, double* lam, double* D, int64_t ldd,
                          int64_t n, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PYROMETHEUS_GB300_H */
