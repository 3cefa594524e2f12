// Mechanism-independent per-state thermochemistry kernels (FP64, sm_103a).
//
// A generated translation unit (pyrometheus_gb300/codegen/cuda.py) defines
// the mechanism sizes and tables below, then includes this file:
//
//   NS, NR         species / reactions
//   NF             falloff reactions (>= 1; a dummy slot when none)
//   NTB            third-body efficiency entries (>= 1)
//   NFRAC          fractional-stoichiometry rows (>= 1)
//   NG             NASA-7 mid-temperature groups
//   MAXSIDE        most species on one side of a reaction
//   BLOCK          threads per block
//   BLOCKS_PER_SM  grid cap of the grid-stride loops
//
// Work split: one thread per thermochemical state (states are independent).
// Every thread of a warp walks the same reaction at the same time, so each
// table read is a uniform constant-cache broadcast; the per-state working
// set (concentrations, Gibbs energies, rate accumulators) lives in a
// per-thread column of shared memory, laid out [quantity][k][BLOCK] so a
// warp's 32 accesses are 32 consecutive doubles (conflict-free).  On GB300
// the FP64 pipe (~2 DFMA/clk/SM) is the bound; table reads, indexing and
// selects issue on other pipes in its shadow.
//
// Formulas follow pyrometheus/chem_expr.py and the generated class of
// pyrometheus/codegen/python.py:106-642 (line references at each function).
#pragma once

#include "pyro_common.cuh"

// PYRO_FAST_EXP (default 1): Tang's table-driven exp of pyro_math.cuh for
// every exponential of the rate evaluation; 0 uses CUDA's exp.
#ifndef PYRO_FAST_EXP
#define PYRO_FAST_EXP 1
#endif
#if PYRO_FAST_EXP
#include "pyro_math.cuh"
#define PEXP(x) pyro_exp(x)
#define PEXP10(x) pyro_exp10(x)
#define PEXP_PRELOAD() PYRO_EXP_PRELOAD()
#define PYRO_STATIC_SMEM PYRO_TABLES_SMEM
#else
#define PYRO_STATIC_SMEM 0
#define PEXP(x) exp(x)
#define PEXP10(x) exp10(x)
#define PEXP_PRELOAD() \
  do {                 \
  } while (0)
#endif

#define RX_KIND_MASK 3
#define RX_ELEMENTARY 0
#define RX_THREE_BODY 1
#define RX_FALLOFF 2
#define RX_REVERSIBLE 4
#define RX_FORM_SHIFT 3
#define RX_TROE 32
#define RX_TROE_T2 64
#define RX_FRACTIONAL 128

// Arrhenius forms (chem_expr.py:310-324)
#define FORM_EXP 0    // exp(ln A + b ln T - Ta / T)
#define FORM_CONST 1  // A            (Ta == 0, b == 0)
#define FORM_POWER 2  // A * T^b      (Ta == 0, integer b, |b| <= 3)

#define GAS_CONSTANT 8314.46261815324
#define IRREVERSIBLE_LOG_KEQ_SLOPE (-0.17364695002734)

namespace pyro {

// Per-thread column of NS doubles: a shared-memory slice (stride BLOCK, the
// threads of a block interleaved) or a thread-private array (stride 1).
template <int STRIDE>
struct ColsT {
  double* base;
  __device__ __forceinline__ double& operator[](int k) const {
    return base[k * STRIDE];
  }
};
using Cols = ColsT<BLOCK>;
using LocalCols = ColsT<1>;

__device__ __forceinline__ Cols col(double* smem, int q) {
  return Cols{smem + (size_t)q * NS * BLOCK + threadIdx.x};
}

// k for one Arrhenius record; x receives the exponent for FORM_EXP.
__device__ __forceinline__ double arrhenius(int form, double p0, double p1,
                                            double p2, double T, double lnT,
                                            double invT, double& x) {
  if (form == FORM_EXP) {
    x = fma(p1, lnT, fma(-p2, invT, p0));
    return PEXP(x);
  }
  x = 0.0;
  if (form == FORM_CONST) return p0;
  const int b = (int)p1;
  const double base = b > 0 ? T : invT;
  double k = p0;
  for (int e = 0; e < (b > 0 ? b : -b); ++e) k *= base;
  return k;
}

__device__ __forceinline__ double ipow_or_pow(double c, double e) {
  if (e == 1.0) return c;
  if (e == 2.0) return c * c;
  return pow(c, e);
}

// NASA-7 coefficients of species k in the range ``up`` selects
// (chem_expr.py:51-57: high range when T > Tmid).  Both ranges are read
// with uniform constant loads and selected, so states on either side of
// Tmid in one warp do not diverge.
struct Nasa {
  int k;
  bool up;
  __device__ __forceinline__ Nasa(int k_, bool up_) : k(k_), up(up_) {}
  __device__ __forceinline__ double operator[](int q) const {
    return up ? k_nasa_hi[k][q] : k_nasa_lo[k][q];
  }
};

// g_k/RT = h/RT - s/R for every species (chem_expr.py:80-117).
template <class CT>
__device__ __forceinline__ void gibbs_all(double T, double lnT, double invT,
                                          CT g) {
  for (int k = 0; k < NS; ++k) {
    const Nasa a(k, T > k_tmid[k]);
    // a0 (1 - ln T) + a5 / T - a6 - T (a1/2 + T (a2/6 + T (a3/12 + T a4/20)))
    g[k] = fma(a[0], 1.0 - lnT, fma(a[5], invT, -a[6])) -
           T * fma(T, fma(T, fma(T, a[4] * (1.0 / 20.0), a[3] * (1.0 / 12.0)),
                          a[2] * (1.0 / 6.0)),
                   a[1] * 0.5);
  }
}

// log K for reaction j (chem_expr.py:274-302; python.py:360-373):
// sum nu'' g - sum nu' g - dnu ln(p0 / RT); irreversible slots hold the
// reference's placeholder -0.17364695002734 T.
template <class CT>
__device__ __forceinline__ double log_keq(int j, int f, double T, double c0,
                                          CT g) {
  if (!(f & RX_REVERSIBLE)) return IRREVERSIBLE_LOG_KEQ_SLOPE * T;
  const int nr = k_rx_nr[j], np = k_rx_np[j];
  double sp = 0.0, sr = 0.0;
  if (f & RX_FRACTIONAL) {
    const int fr = k_rx_frac[j];
    for (int a = 0; a < MAXSIDE; ++a) {
      if (a < np)
        sp = fma(k_frac[fr][MAXSIDE + a], g[k_rx_sp[j][MAXSIDE + a]], sp);
      if (a < nr) sr = fma(k_frac[fr][a], g[k_rx_sp[j][a]], sr);
    }
  } else {
    for (int a = 0; a < MAXSIDE; ++a) {
      if (a < np) {
        const int nu = k_rx_nu[j][MAXSIDE + a];
        const double gv = g[k_rx_sp[j][MAXSIDE + a]];
        sp += nu == 1 ? gv : (double)nu * gv;
      }
      if (a < nr) {
        const int nu = k_rx_nu[j][a];
        const double gv = g[k_rx_sp[j][a]];
        sr += nu == 1 ? gv : (double)nu * gv;
      }
    }
  }
  const double dnu = k_rx_dnu[j];
  double lk = sp - sr;
  if (dnu != 0.0) lk -= dnu * c0;
  return lk;
}

// Forward/reverse rates of progress of reaction j.
//   kf: forward rate coefficient with [M] and falloff folded in
//       (python.py:399-473)
//   rf = kf prod c^ord'  (orders paired positionally, chem_expr.py:436-446)
//   rr = kf exp(log K) prod c^nu''  (0 when irreversible or !want_rev)
// With dlnk_dlnm, also d ln kf / d ln [M] (0 elementary, 1 three-body,
// 1/(1 + Pr) + d ln F / d ln Pr falloff; the reverse coefficient shares it).
template <class CT>
__device__ __forceinline__ void reaction_rates(int j, double T, double lnT,
                                               double invT, double c0,
                                               double ctot, CT c, CT g,
                                               bool want_rev, double& kf,
                                               double& rf, double& rr,
                                               double* dlnk_dlnm = nullptr) {
  const int f = k_rx_flags[j];
  const int kind = f & RX_KIND_MASK;
  const int form = (f >> RX_FORM_SHIFT) & 3;
  double m = 1.0;
  if (kind != RX_ELEMENTARY) {
    // [M] = default * sum_k c_k + sum_listed (eff_k - default) c_k
    // (chem_expr.py:327-345)
    const double d = k_rx_defeff[j];
    m = d == 0.0 ? 0.0 : (d == 1.0 ? ctot : d * ctot);
    for (int t = k_rx_tb[j]; t < k_rx_tb[j + 1]; ++t)
      m = fma(k_tb_de[t], c[k_tb_idx[t]], m);
  }
  double x = 0.0;
  bool exp_form = false;
  if (kind == RX_FALLOFF) {
    // k = k_hi F Pr / (1 + Pr), Pr = [M] k_lo / k_hi (python.py:399-450)
    const int s = k_rx_fo[j];
    double xh, xl;
    const double k_hi = arrhenius(form, k_rx_rate[j][0], k_rx_rate[j][1],
                                  k_rx_rate[j][2], T, lnT, invT, xh);
    const double k_lo =
        arrhenius(k_fo_lowform[s], k_fo_low[s][0], k_fo_low[s][1],
                  k_fo_low[s][2], T, lnT, invT, xl);
    const double pr = m * k_lo / k_hi;
    double blend = 1.0, dlnf = 0.0;
    if (f & RX_TROE) {
      // log10 Fcent, Troe broadening (chem_expr.py:348-420)
      double fsum = k_fo_troe[s][0] * PEXP(T * k_fo_troe[s][1]) +
                    k_fo_troe[s][2] * PEXP(T * k_fo_troe[s][3]);
      if (f & RX_TROE_T2) fsum += PEXP(k_fo_troe[s][4] * invT);
      const double log_fc = log10(fsum);
      double fac = -1.0 / 0.14;
      if (pr > 0.0) {
        const double xx = log10(pr) + (-0.4 - 0.67 * log_fc);
        const double den = 0.75 - 1.27 * log_fc;
        const double dd = den - 0.14 * xx;
        fac = xx / dd;
        if (dlnk_dlnm) {
          // d log10 F / d log10 Pr = -2 log10 Fcent f / (1 + f^2)^2 df/dxx
          const double q = 1.0 + fac * fac;
          dlnf = -2.0 * log_fc * fac / (q * q) * (den / (dd * dd));
        }
      }
      blend = PEXP10(log_fc / (1.0 + fac * fac));
    }
    kf = k_hi * (blend * pr / (1.0 + pr));
    if (dlnk_dlnm) *dlnk_dlnm = 1.0 / (1.0 + pr) + dlnf;
  } else {
    const double ek = arrhenius(form, k_rx_rate[j][0], k_rx_rate[j][1],
                                k_rx_rate[j][2], T, lnT, invT, x);
    exp_form = form == FORM_EXP;
    kf = kind == RX_THREE_BODY ? ek * m : ek;
    if (dlnk_dlnm) *dlnk_dlnm = kind == RX_THREE_BODY ? 1.0 : 0.0;
  }
  const int nr = k_rx_nr[j], np = k_rx_np[j];
  const bool frac = (f & RX_FRACTIONAL) != 0;
  const int fr = k_rx_frac[j];
  double pf = 1.0;
  for (int a = 0; a < MAXSIDE; ++a) {
    if (a < nr) {
      const double cv = c[k_rx_sp[j][a]];
      const double e =
          frac ? k_frac[fr][2 * MAXSIDE + a] : (double)k_rx_ord[j][a];
      pf *= ipow_or_pow(cv, e);
    }
  }
  rf = kf * pf;
  rr = 0.0;
  if (want_rev && (f & RX_REVERSIBLE)) {
    const double lk = log_keq(j, f, T, c0, g);
    double kr;
    if (exp_form) {
      // k_r = exp(ln k_f + log K) [* M]: reuses the forward exponent
      kr = PEXP(x + lk);
      if (kind == RX_THREE_BODY) kr *= m;
    } else {
      kr = kf * PEXP(lk);
    }
    double pv = 1.0;
    for (int a = 0; a < MAXSIDE; ++a) {
      if (a < np) {
        const double cv = c[k_rx_sp[j][MAXSIDE + a]];
        const double e = frac ? k_frac[fr][MAXSIDE + a]
                              : (double)k_rx_nu[j][MAXSIDE + a];
        pv *= ipow_or_pow(cv, e);
      }
    }
    rr = kr * pv;
  }
}

// Scatter a rate into per-species accumulators with weights -nu' / +nu''.
template <class CT>
__device__ __forceinline__ void scatter_net(int j, double q, CT w) {
  const int f = k_rx_flags[j];
  const int nr = k_rx_nr[j], np = k_rx_np[j];
  if (f & RX_FRACTIONAL) {
    const int fr = k_rx_frac[j];
    for (int a = 0; a < MAXSIDE; ++a) {
      if (a < nr) {
        double& t = w[k_rx_sp[j][a]];
        t = fma(-k_frac[fr][a], q, t);
      }
      if (a < np) {
        double& t = w[k_rx_sp[j][MAXSIDE + a]];
        t = fma(k_frac[fr][MAXSIDE + a], q, t);
      }
    }
    return;
  }
  for (int a = 0; a < MAXSIDE; ++a) {
    if (a < nr) {
      const int nu = k_rx_nu[j][a];
      double& t = w[k_rx_sp[j][a]];
      t = nu == 1 ? t - q : fma(-(double)nu, q, t);
    }
    if (a < np) {
      const int nu = k_rx_nu[j][MAXSIDE + a];
      double& t = w[k_rx_sp[j][MAXSIDE + a]];
      t = nu == 1 ? t + q : fma((double)nu, q, t);
    }
  }
}

// creation += nu'' rf + nu' rr ; destruction += nu' rf + nu'' rr
// (chem_expr.py:525-567)
template <class CT>
__device__ __forceinline__ void scatter_cd(int j, double rf, double rr,
                                           CT cd, CT dd) {
  const int f = k_rx_flags[j];
  const int nr = k_rx_nr[j], np = k_rx_np[j];
  const bool frac = (f & RX_FRACTIONAL) != 0;
  const int fr = k_rx_frac[j];
  for (int a = 0; a < MAXSIDE; ++a) {
    if (a < nr) {
      const double nu = frac ? k_frac[fr][a] : (double)k_rx_nu[j][a];
      const int k = k_rx_sp[j][a];
      dd[k] = fma(nu, rf, dd[k]);
      cd[k] = fma(nu, rr, cd[k]);
    }
    if (a < np) {
      const double nu =
          frac ? k_frac[fr][MAXSIDE + a] : (double)k_rx_nu[j][MAXSIDE + a];
      const int k = k_rx_sp[j][MAXSIDE + a];
      cd[k] = fma(nu, rf, cd[k]);
      dd[k] = fma(nu, rr, dd[k]);
    }
  }
}

// Per-state prologue: ln T, 1/T, ln(p0/RT), concentrations, total
// concentration (python.py:272-277: c_k = (1/W_k) rho Y_k).
struct StateScalars {
  double T, lnT, invT, c0, ctot;
};

template <class CT>
__device__ __forceinline__ StateScalars state_from_mass(
    double T, double rho, const double* __restrict__ Y, int64_t ldy,
    int64_t i, CT c) {
  StateScalars s;
  s.T = T;
  s.lnT = log(T);
  s.invT = 1.0 / T;
  s.c0 = LOG_P0_OVER_R - s.lnT;
  double ctot = 0.0;
  for (int k = 0; k < NS; ++k) {
    const double v = k_inv_mw[k] * rho * __ldg(Y + (int64_t)k * ldy + i);
    c[k] = v;
    ctot += v;
  }
  s.ctot = ctot;
  return s;
}

__device__ __forceinline__ StateScalars state_from_conc(
    double T, const double* __restrict__ conc, int64_t ldc, int64_t i,
    Cols c, bool load) {
  StateScalars s;
  s.T = T;
  s.lnT = log(T);
  s.invT = 1.0 / T;
  s.c0 = LOG_P0_OVER_R - s.lnT;
  double ctot = 0.0;
  if (load) {
    for (int k = 0; k < NS; ++k) {
      const double v = __ldg(conc + (int64_t)k * ldc + i);
      c[k] = v;
      ctot += v;
    }
  }
  s.ctot = ctot;
  return s;
}

// Net production rates of one state into w (python.py:486-495).
template <class CT>
__device__ __forceinline__ void production_rates(const StateScalars& s,
                                                 CT c, CT g, CT w) {
  gibbs_all(s.T, s.lnT, s.invT, g);
  for (int k = 0; k < NS; ++k) w[k] = 0.0;
  for (int j = 0; j < NR; ++j) {
    double kf, rf, rr;
    reaction_rates(j, s.T, s.lnT, s.invT, s.c0, s.ctot, c, g, true, kf, rf,
                   rr);
    scatter_net(j, rf - rr, w);
  }
}

// Temperature from mixture energy or enthalpy (python.py:375-396): Newton
// dT = (target - e(T)) / cv(T) per state, stop at |dT| < tol.  The
// mass-weighted NASA-7 coefficients are folded once, so an iteration costs
// one degree-5 polynomial per mid-temperature group instead of S of them.
__device__ __forceinline__ bool temperature_newton(
    double target, double t0, const double* __restrict__ Y, int64_t ldy,
    int64_t i, bool do_energy, double tol, int max_iter, double& Tout) {
  double P[NG][2][6];
  double wsum = 0.0;
#pragma unroll
  for (int gq = 0; gq < NG; ++gq) {
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int q = 0; q < 6; ++q) P[gq][r][q] = 0.0;
    for (int t = k_grp_start[gq]; t < k_grp_start[gq + 1]; ++t) {
      const int k = k_grp_sp[t];
      const double wk = __ldg(Y + (int64_t)k * ldy + i) * k_inv_mw[k];
      wsum += wk;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        P[gq][0][q] = fma(wk, k_nasa_hi[k][q], P[gq][0][q]);
        P[gq][1][q] = fma(wk, k_nasa_lo[k][q], P[gq][1][q]);
      }
    }
  }
  const double tgt = target * (1.0 / GAS_CONSTANT);
  double T = t0;
  for (int it = 0; it < max_iter; ++it) {
    double cp = 0.0, h = 0.0;
#pragma unroll
    for (int gq = 0; gq < NG; ++gq) {
      const bool up = T > k_grp_tmid[gq];
      double p[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) p[q] = up ? P[gq][0][q] : P[gq][1][q];
      // cp/R = sum p_i T^i ; h/R = p5 + sum p_i T^(i+1) / (i+1)
      cp += fma(T, fma(T, fma(T, fma(T, p[4], p[3]), p[2]), p[1]), p[0]);
      h += fma(T, fma(T, fma(T, fma(T, fma(T, p[4] * 0.2, p[3] * 0.25),
                                          p[2] * (1.0 / 3.0)),
                                  p[1] * 0.5),
                          p[0]),
               p[5]);
    }
    if (do_energy) {
      cp -= wsum;
      h -= wsum * T;
    }
    const double dT = (tgt - h) / cp;
    T += dT;
    if (fabs(dT) < tol) {
      Tout = T;
      return true;
    }
  }
  Tout = T;
  return false;
}

}  // namespace pyro

// ------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------

#define PYRO_LOOP(i)                                                       \
  for (int64_t i = (int64_t)blockIdx.x * BLOCK + threadIdx.x; i < n;       \
       i += (int64_t)gridDim.x * BLOCK)

// species NASA-7 properties (python.py:313-358); which:
// 0 cp/R, 1 h/RT, 2 s/R, 3 g/RT, 4 d(cp/R)/dT, 5 d(h/RT)/dT, 6 d(s/R)/dT
__global__ void __launch_bounds__(BLOCK)
    k_species_prop(int which, const double* __restrict__ Tp, int64_t t_inc,
                   double* __restrict__ out, int64_t ldo, int64_t n) {
  PYRO_LOOP(i) {
    const double T = pyro_ld(Tp, t_inc, i);
    const double lnT = log(T), invT = 1.0 / T;
    for (int k = 0; k < NS; ++k) {
      const pyro::Nasa a(k, T > k_tmid[k]);
      double v;
      switch (which) {
        case 0:
          v = fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
          break;
        case 1:
          v = fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                                a[2] * (1.0 / 3.0)),
                        a[1] * 0.5),
                  a[0]) +
              a[5] * invT;
          break;
        case 2:
          v = fma(a[0], lnT,
                  fma(T, fma(T, fma(T, fma(T, a[4] * 0.25, a[3] * (1.0 / 3.0)),
                                    a[2] * 0.5),
                          a[1]),
                      a[6]));
          break;
        case 3:
          v = fma(a[0], 1.0 - lnT, fma(a[5], invT, -a[6])) -
              T * fma(T, fma(T, fma(T, a[4] * (1.0 / 20.0),
                                    a[3] * (1.0 / 12.0)),
                             a[2] * (1.0 / 6.0)),
                      a[1] * 0.5);
          break;
        case 4:
          v = fma(T, fma(T, 4.0 * a[4], 3.0 * a[3]), 2.0 * a[2]) * T + a[1];
          break;
        case 5:
          v = fma(T, fma(T, a[4] * 0.8, a[3] * 0.75), a[2] * (2.0 / 3.0)) * T +
              a[1] * 0.5 - a[5] * invT * invT;
          break;
        default:
          v = a[0] * invT + fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]);
          break;
      }
      out[(int64_t)k * ldo + i] = v;
    }
  }
}

// mixture properties (python.py:248-311); which:
// 0 W_mix, 1 R/W_mix, 2 cp, 3 cv, 4 h, 5 e (mass), 6 rho from p=aux,
// 7 p from rho=aux
__global__ void __launch_bounds__(BLOCK)
    k_mixture_prop(int which, const double* __restrict__ Tp, int64_t t_inc,
                   const double* __restrict__ Y, int64_t ldy,
                   const double* __restrict__ aux, int64_t aux_inc,
                   double* __restrict__ out, int64_t n) {
  PYRO_LOOP(i) {
    double inv_mmw = 0.0;
    for (int k = 0; k < NS; ++k)
      inv_mmw = fma(k_inv_mw[k], __ldg(Y + (int64_t)k * ldy + i), inv_mmw);
    double v;
    if (which == 0) {
      v = 1.0 / inv_mmw;
    } else if (which == 1) {
      v = GAS_CONSTANT * inv_mmw;
    } else {
      const double T = pyro_ld(Tp, t_inc, i);
      if (which == 6) {
        v = pyro_ld(aux, aux_inc, i) * (1.0 / inv_mmw) / (GAS_CONSTANT * T);
      } else if (which == 7) {
        v = pyro_ld(aux, aux_inc, i) * (GAS_CONSTANT * T) / (1.0 / inv_mmw);
      } else {
        const double invT = 1.0 / T;
        double acc = 0.0;
        for (int k = 0; k < NS; ++k) {
          const pyro::Nasa a(k, T > k_tmid[k]);
          const double wk = __ldg(Y + (int64_t)k * ldy + i) * k_inv_mw[k];
          double p;
          if (which <= 3)
            p = fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
          else
            p = fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                                  a[2] * (1.0 / 3.0)),
                          a[1] * 0.5),
                    a[0]) +
                a[5] * invT;
          acc = fma(wk, p, acc);
        }
        if (which == 3 || which == 5) acc -= inv_mmw;
        v = which <= 3 ? GAS_CONSTANT * acc : GAS_CONSTANT * T * acc;
      }
    }
    out[i] = v;
  }
}

// concentrations (which 0: (1/W) rho Y, python.py:272-277) and mole
// fractions (which 1: (1/W) Y W_mix, python.py:279-285); aux = rho or W_mix
__global__ void __launch_bounds__(BLOCK)
    k_species_scale(int which, const double* __restrict__ aux,
                    int64_t aux_inc, const double* __restrict__ Y,
                    int64_t ldy, double* __restrict__ out, int64_t ldo,
                    int64_t n) {
  PYRO_LOOP(i) {
    const double a = pyro_ld(aux, aux_inc, i);
    for (int k = 0; k < NS; ++k) {
      const double y = __ldg(Y + (int64_t)k * ldy + i);
      out[(int64_t)k * ldo + i] = which == 0 ? k_inv_mw[k] * a * y
                                             : k_inv_mw[k] * y * a;
    }
  }
}

// per-reaction quantities from (T, concentrations); mode:
// 0 log K (python.py:360-373), 1 k_fwd (python.py:453-473),
// 2 net rate of progress (python.py:475-484), 3 forward (497-504),
// 4 reverse (506-515)
__global__ void __launch_bounds__(BLOCK)
    k_reaction_quantity(int mode, const double* __restrict__ Tp,
                        int64_t t_inc, const double* __restrict__ conc,
                        int64_t ldc, double* __restrict__ out, int64_t ldo,
                        int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  const pyro::Cols c = pyro::col(smem, 0), g = pyro::col(smem, 1);
  PYRO_LOOP(i) {
    const double T = pyro_ld(Tp, t_inc, i);
    const pyro::StateScalars s =
        pyro::state_from_conc(T, conc, ldc, i, c, mode != 0);
    if (mode == 0 || mode == 2 || mode == 4)
      pyro::gibbs_all(s.T, s.lnT, s.invT, g);
    for (int j = 0; j < NR; ++j) {
      double v;
      if (mode == 0) {
        v = pyro::log_keq(j, k_rx_flags[j], s.T, s.c0, g);
      } else {
        double kf, rf, rr;
        pyro::reaction_rates(j, s.T, s.lnT, s.invT, s.c0, s.ctot, c, g,
                             mode == 2 || mode == 4, kf, rf, rr);
        v = mode == 1 ? kf : (mode == 2 ? rf - rr : (mode == 3 ? rf : rr));
      }
      out[(int64_t)j * ldo + i] = v;
    }
  }
}

// net production rates (python.py:486-495): the hot path
__global__ void __launch_bounds__(BLOCK)
    k_net_production_rates(const double* __restrict__ rhop, int64_t rho_inc,
                           const double* __restrict__ Tp, int64_t t_inc,
                           const double* __restrict__ Y, int64_t ldy,
                           double* __restrict__ wdot, int64_t ldw,
                           int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  const pyro::Cols c = pyro::col(smem, 0), g = pyro::col(smem, 1),
                   w = pyro::col(smem, 2);
  PYRO_LOOP(i) {
    const pyro::StateScalars s = pyro::state_from_mass(
        pyro_ld(Tp, t_inc, i), pyro_ld(rhop, rho_inc, i), Y, ldy, i, c);
    pyro::production_rates(s, c, g, w);
    for (int k = 0; k < NS; ++k) wdot[(int64_t)k * ldw + i] = w[k];
  }
}

// creation and destruction rates (python.py:517-562)
__global__ void __launch_bounds__(BLOCK)
    k_creation_destruction(const double* __restrict__ rhop, int64_t rho_inc,
                           const double* __restrict__ Tp, int64_t t_inc,
                           const double* __restrict__ Y, int64_t ldy,
                           double* __restrict__ cdot,
                           double* __restrict__ ddot, int64_t ldo,
                           int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  const pyro::Cols c = pyro::col(smem, 0), g = pyro::col(smem, 1),
                   cd = pyro::col(smem, 2), dd = pyro::col(smem, 3);
  PYRO_LOOP(i) {
    const pyro::StateScalars s = pyro::state_from_mass(
        pyro_ld(Tp, t_inc, i), pyro_ld(rhop, rho_inc, i), Y, ldy, i, c);
    pyro::gibbs_all(s.T, s.lnT, s.invT, g);
    for (int k = 0; k < NS; ++k) {
      cd[k] = 0.0;
      dd[k] = 0.0;
    }
    for (int j = 0; j < NR; ++j) {
      double kf, rf, rr;
      pyro::reaction_rates(j, s.T, s.lnT, s.invT, s.c0, s.ctot, c, g, true,
                           kf, rf, rr);
      pyro::scatter_cd(j, rf, rr, cd, dd);
    }
    for (int k = 0; k < NS; ++k) {
      if (cdot) cdot[(int64_t)k * ldo + i] = cd[k];
      if (ddot) ddot[(int64_t)k * ldo + i] = dd[k];
    }
  }
}

// temperature Newton (python.py:375-396)
__global__ void __launch_bounds__(BLOCK)
    k_temperature(const double* __restrict__ target, int64_t target_inc,
                  const double* __restrict__ t0, int64_t t0_inc,
                  const double* __restrict__ Y, int64_t ldy, int do_energy,
                  double tol, int max_iter, double* __restrict__ Tout,
                  int* __restrict__ fail_count, int64_t n) {
  PYRO_LOOP(i) {
    double T;
    const bool ok = pyro::temperature_newton(
        pyro_ld(target, target_inc, i), pyro_ld(t0, t0_inc, i), Y, ldy, i,
        do_energy != 0, tol, max_iter, T);
    Tout[i] = T;
    if (!ok && fail_count) atomicAdd(fail_count, 1);
  }
}

// fused state step: rho = p W / (R T); net production rates; temperature
// from energy/enthalpy (the chain of reactors.py:115-123 and
// flamelets/equations.py:313-359)
__global__ void __launch_bounds__(BLOCK)
    k_fused_step(const double* __restrict__ Pp, int64_t p_inc,
                 const double* __restrict__ Tp, int64_t t_inc,
                 const double* __restrict__ Y, int64_t ldy,
                 const double* __restrict__ target, int64_t target_inc,
                 const double* __restrict__ t0, int64_t t0_inc, int do_energy,
                 double tol, int max_iter, double* __restrict__ wdot,
                 int64_t ldw, double* __restrict__ Tout,
                 int* __restrict__ fail_count, int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  const pyro::Cols c = pyro::col(smem, 0), g = pyro::col(smem, 1),
                   w = pyro::col(smem, 2);
  PYRO_LOOP(i) {
    const double T = pyro_ld(Tp, t_inc, i);
    double inv_mmw = 0.0;
    for (int k = 0; k < NS; ++k)
      inv_mmw = fma(k_inv_mw[k], __ldg(Y + (int64_t)k * ldy + i), inv_mmw);
    const double rho =
        pyro_ld(Pp, p_inc, i) * (1.0 / inv_mmw) / (GAS_CONSTANT * T);
    const pyro::StateScalars s = pyro::state_from_mass(T, rho, Y, ldy, i, c);
    pyro::production_rates(s, c, g, w);
    for (int k = 0; k < NS; ++k) wdot[(int64_t)k * ldw + i] = w[k];
    double Tn;
    const bool ok = pyro::temperature_newton(
        pyro_ld(target, target_inc, i), pyro_ld(t0, t0_inc, i), Y, ldy, i,
        do_energy != 0, tol, max_iter, Tn);
    Tout[i] = Tn;
    if (!ok && fail_count) atomicAdd(fail_count, 1);
  }
}
