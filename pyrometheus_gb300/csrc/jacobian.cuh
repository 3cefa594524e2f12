// Analytic Jacobian and vector-Jacobian product of the adiabatic
// constant-pressure reactor source (FP64, sm_103a).
//
// State x = (T, Y_1..Y_S), source f = (dT/dt, dY_1/dt..dY_S/dt):
//   rho = p / (R T sigma),  sigma = sum_k Y_k / W_k,  c_k = rho Y_k / W_k,
//   dY_k/dt = W_k w_k / rho,
//   dT/dt   = -Q / (rho cp),  Q = sum_k H_k w_k,  H_k = R T (h/RT)_k,
//   cp = R sum_k (Y_k/W_k) (cp/R)_k,
// with w_k the net production rates (python.py:486-495).  This is the
// right-hand side the reference differentiates with jax.jacfwd for its
// reactors and flamelets (examples/free_flame/reactors.py:115-125,
// flamelets/equations.py:124-129, 361-389); here the derivative is written
// out by hand:
//
//   per reaction:  q = kf prod c^o' - kr prod c^nu'',  with dq/dT at fixed c
//   (Arrhenius exponent derivatives b/T + Ta/T^2, d log K/dT =
//   (dnu - sum nu'' h/RT + sum nu' h/RT) / T, Troe blending through
//   log10 Fcent(T) and log10 Pr), dq/dM (third body / falloff) and the
//   mass-action dq/dc_m;
//   chain rule through c(T, Y) and rho(T, Y), then the dT/dt row.
//
// k_reactor_jacobian: a group of one warp per state (two warps for large
// mechanisms).  Lanes take reactions in generated blocks of one kind per
// warp and round (sorted by reversibility and side sizes within), so a
// warp's lanes run the same code path and trip counts; the
// tables they index with different reactions or species are global-memory
// copies read through L1 (the constant cache would serialise the 32
// different addresses).  Each lane writes, per slot of its reaction, the
// partial derivative of the rate of progress with respect to that slot's
// concentration (and dq/dM) into a per-warp shared-memory vector D.  The
// S x S block dw/dc is then built in the interior of the state's own output
// block from a generated update list: entries (element, source in D,
// stoichiometric coefficient) sorted by element and split into 32 runs of
// equal length, one per lane, so every element is summed by one lane in a
// fixed order and stored once -- no atomics and no divergent trip counts.
// The third-body default efficiency contributes a rank-1 term added in the
// assembly instead of S entries per reaction.  Shared memory holds per-warp
// vectors only (about 21 KB per warp at 53 species / 325 reactions).  The
// output is written row by row, 32 consecutive doubles per warp store.
//
// k_reactor_vjp: one thread per state, reverse accumulation.  Each reaction
// gets one scalar adjoint mu_r = sum_k lambda_k nu_kr, so the cost is a
// small multiple of the production rates and J is never formed.
#pragma once

#include "kinetics.cuh"

namespace pyro {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// d(exponent)/dT of an Arrhenius record (FORM_EXP: b/T + Ta/T^2).
__device__ __forceinline__ double darr_dT(int form, double b, double ta,
                                          double invT) {
  if (form == FORM_EXP) return fma(ta, invT, b) * invT;
  if (form == FORM_CONST) return 0.0;
  return b * invT;
}

struct RxnDeriv {
  double q;      // net rate of progress
  double dqdT;   // at fixed concentrations
  double dqdM;   // w.r.t. the third-body concentration (0 if none)
  double kf;     // forward rate coefficient ([M], falloff folded in)
  double kr;     // reverse rate coefficient (0 if irreversible)
};

// d(prod_b c_b^e_b)/dc at position a of a reaction side.
template <class CT>
__device__ __forceinline__ double dprod(int j, int side, int a, int cnt,
                                        bool frac, CT c) {
  const int base = side ? MAXSIDE : 0;
  double others = 1.0;
  double ea = 1.0;
  for (int b = 0; b < MAXSIDE; ++b) {
    if (b >= cnt) break;
    const double cv = c[k_rx_sp[j][base + b]];
    double e;
    if (side == 0)
      e = frac ? k_frac[k_rx_frac[j]][2 * MAXSIDE + b] : (double)k_rx_ord[j][b];
    else
      e = frac ? k_frac[k_rx_frac[j]][MAXSIDE + b]
               : (double)k_rx_nu[j][MAXSIDE + b];
    if (b == a)
      ea = e;
    else
      others *= ipow_or_pow(cv, e);
  }
  const double cm = c[k_rx_sp[j][base + a]];
  double d;
  if (ea == 1.0)
    d = 1.0;
  else if (ea == 2.0)
    d = 2.0 * cm;
  else
    d = ea * pow(cm, ea - 1.0);
  return d * others;
}

// Falloff rate coefficient and its derivatives (Lindemann, or Troe when
// `troe`): kf = k_hi F Pr / (1 + Pr), Pr = m k_lo / k_hi, log10 F =
// log10 Fcent / (1 + f^2), f = x / (n - 0.14 x), x = log10 Pr - 0.4 -
// 0.67 log10 Fcent, n = 0.75 - 1.27 log10 Fcent (python.py's falloff
// blending); returns kf, d ln kf / dT at fixed m (dxh, dxl: the exponent
// derivatives of k_hi, k_lo) and d kf / dm.  Five divisions (reciprocals
// reused) and the table logarithm read through L1.
struct FalloffDeriv {
  double kf, dlnkf, dkfdM;
};

__device__ __forceinline__ FalloffDeriv falloff_deriv(
    bool troe, bool troe_t2, double a0, double a1, double a2, double a3,
    double a4, double T, double invT, double m, double k_hi, double k_lo,
    double dxh, double dxl) {
  const double pr = m * k_lo / k_hi;
  double blend = 1.0, dlnF_dT = 0.0, phi_x = 0.0;
  if (troe) {
    const double ln10 = 2.302585092994045684;
    const double e3 = PEXP(T * a1);
    const double e1 = PEXP(T * a3);
    double fsum = a0 * e3 + a2 * e1;
    double dfsum = a0 * a1 * e3 + a2 * a3 * e1;
    if (troe_t2) {
      const double e2 = PEXP(a4 * invT);
      fsum += e2;
      dfsum -= a4 * invT * invT * e2;
    }
    const double L = pyro_log10_g(fsum);
    const double dL = dfsum / (fsum * ln10);
    double fac = -1.0 / 0.14, dfac = 0.0, fx = 0.0;
    if (pr > 0.0) {
      const double xx = pyro_log10_g(pr) + (-0.4 - 0.67 * L);
      const double nn = 0.75 - 1.27 * L;
      const double iden = 1.0 / (nn - 0.14 * xx);
      fac = xx * iden;
      fx = nn * iden * iden;
      const double fn = -fac * iden;
      const double dxx = (dxl - dxh) * (1.0 / ln10) - 0.67 * dL;
      dfac = fx * dxx + fn * (-1.27 * dL);
    }
    const double iopf = 1.0 / (1.0 + fac * fac);
    blend = PEXP10(L * iopf);
    const double g2 = 2.0 * L * fac * iopf * iopf;
    dlnF_dT = ln10 * (dL * iopf - g2 * dfac);
    phi_x = -g2 * fx;
  }
  const double i1pr = 1.0 / (1.0 + pr);
  FalloffDeriv o;
  o.kf = k_hi * (blend * pr * i1pr);
  o.dlnkf = dxh + dlnF_dT + (dxl - dxh) * i1pr;
  o.dkfdM = blend * k_lo * i1pr * (phi_x + i1pr);
  return o;
}

// Net rate, its temperature and third-body derivatives, and the rate
// coefficients of reaction j.  h: column of h/RT.
template <class CT>
__device__ __forceinline__ RxnDeriv reaction_deriv(int j,
                                                   const StateScalars& s,
                                                   CT c, CT g, CT h) {
  const double T = s.T, lnT = s.lnT, invT = s.invT;
  const int f = k_rx_flags[j];
  const int kind = f & RX_KIND_MASK;
  const int form = (f >> RX_FORM_SHIFT) & 3;
  double m = 1.0;
  if (kind != RX_ELEMENTARY) {
    const double d = k_rx_defeff[j];
    m = d == 0.0 ? 0.0 : (d == 1.0 ? s.ctot : d * s.ctot);
    for (int t = k_rx_tb[j]; t < k_rx_tb[j + 1]; ++t)
      m = fma(k_tb_de[t], c[k_tb_idx[t]], m);
  }
  RxnDeriv out;
  double x = 0.0, dlnkf = 0.0, dkfdM = 0.0, ek = 0.0;
  bool exp_form = false;
  if (kind == RX_FALLOFF) {
    const int sl = k_rx_fo[j];
    const int lform = k_fo_lowform[sl];
    double xh, xl;
    const double k_hi = arrhenius(form, k_rx_rate[j][0], k_rx_rate[j][1],
                                  k_rx_rate[j][2], T, lnT, invT, xh);
    const double k_lo = arrhenius(lform, k_fo_low[sl][0], k_fo_low[sl][1],
                                  k_fo_low[sl][2], T, lnT, invT, xl);
    const double dxh = darr_dT(form, k_rx_rate[j][1], k_rx_rate[j][2], invT);
    const double dxl = darr_dT(lform, k_fo_low[sl][1], k_fo_low[sl][2], invT);
    const FalloffDeriv fd = falloff_deriv(
        (f & RX_TROE) != 0, (f & RX_TROE_T2) != 0, k_fo_troe[sl][0],
        k_fo_troe[sl][1], k_fo_troe[sl][2], k_fo_troe[sl][3],
        k_fo_troe[sl][4], T, invT, m, k_hi, k_lo, dxh, dxl);
    out.kf = fd.kf;
    dlnkf = fd.dlnkf;
    dkfdM = fd.dkfdM;
  } else {
    ek = arrhenius(form, k_rx_rate[j][0], k_rx_rate[j][1], k_rx_rate[j][2], T,
                   lnT, invT, x);
    exp_form = form == FORM_EXP;
    dlnkf = darr_dT(form, k_rx_rate[j][1], k_rx_rate[j][2], invT);
    if (kind == RX_THREE_BODY) {
      out.kf = ek * m;
      dkfdM = ek;
    } else {
      out.kf = ek;
    }
  }
  const int nr = k_rx_nr[j], np = k_rx_np[j];
  const bool frac = (f & RX_FRACTIONAL) != 0;
  const int fr = k_rx_frac[j];
  double pf = 1.0;
  for (int a = 0; a < MAXSIDE; ++a) {
    if (a >= nr) break;
    const double e = frac ? k_frac[fr][2 * MAXSIDE + a] : (double)k_rx_ord[j][a];
    pf *= ipow_or_pow(c[k_rx_sp[j][a]], e);
  }
  out.kr = 0.0;
  double pv = 0.0, dlnkr = 0.0, dkrdM = 0.0;
  if (f & RX_REVERSIBLE) {
    const double lk = log_keq(j, f, T, s.c0, g);
    // d log K / dT = (dnu - sum nu'' h/RT + sum nu' h/RT) / T
    double dh = 0.0, dnu = k_rx_dnu[j];
    pv = 1.0;
    for (int a = 0; a < MAXSIDE; ++a) {
      if (a < np) {
        const int k = k_rx_sp[j][MAXSIDE + a];
        const double nu =
            frac ? k_frac[fr][MAXSIDE + a] : (double)k_rx_nu[j][MAXSIDE + a];
        dh = fma(nu, h[k], dh);
        pv *= ipow_or_pow(c[k], nu);
      }
      if (a < nr) {
        const double nu = frac ? k_frac[fr][a] : (double)k_rx_nu[j][a];
        dh = fma(-nu, h[k_rx_sp[j][a]], dh);
      }
    }
    const double dlk = (dnu - dh) * invT;
    if (exp_form) {
      const double ekr = PEXP(x + lk);
      out.kr = kind == RX_THREE_BODY ? ekr * m : ekr;
      dkrdM = kind == RX_THREE_BODY ? ekr : 0.0;
    } else {
      const double eK = PEXP(lk);
      out.kr = out.kf * eK;
      dkrdM = dkfdM * eK;
    }
    dlnkr = dlnkf + dlk;
  }
  out.q = out.kf * pf - out.kr * pv;
  out.dqdT = out.kf * dlnkf * pf - out.kr * dlnkr * pv;
  out.dqdM = dkfdM * pf - dkrdM * pv;
  return out;
}

// Signed stoichiometric weight (-nu' for a reactant slot, +nu'' for a
// product slot) of slot `pos` of reaction j.
__device__ __forceinline__ double slot_nu(int j, int pos) {
  const int f = k_rx_flags[j];
  const bool frac = (f & RX_FRACTIONAL) != 0;
  if (pos < MAXSIDE)
    return -(frac ? k_frac[k_rx_frac[j]][pos] : (double)k_rx_nu[j][pos]);
  return frac ? k_frac[k_rx_frac[j]][pos] : (double)k_rx_nu[j][pos];
}

// Per-state thermo of one species: cp/R, h/RT, g/RT, d(cp/R)/dT.
struct SpThermo {
  double cp, h, g, dcp;
};

__device__ __forceinline__ SpThermo species_thermo(int k, double T,
                                                   double lnT, double invT) {
  const Nasa a(k, T > k_tmid[k]);
  SpThermo t;
  t.cp = fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
  t.h = fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                          a[2] * (1.0 / 3.0)),
                  a[1] * 0.5),
            a[0]) +
        a[5] * invT;
  t.g = fma(a[0], 1.0 - lnT, fma(a[5], invT, -a[6])) -
        T * fma(T, fma(T, fma(T, a[4] * (1.0 / 20.0), a[3] * (1.0 / 12.0)),
                       a[2] * (1.0 / 6.0)),
                a[1] * 0.5);
  t.dcp = fma(T, fma(T, 4.0 * a[4], 3.0 * a[3]), 2.0 * a[2]) * T + a[1];
  return t;
}

}  // namespace pyro

namespace pyro {

// Rate-of-progress derivatives of reaction qq (permuted numbering) from the
// global Jacobian tables: q, dq/dT at fixed c, dq/dM, and per slot s of the
// reaction dq/dc_{sp(s)} into D[s]; dq/dM goes to D[NSLOT + qq].  Also
// Hq = sum over slots of nu h/RT, and Qc = sum_m dq/dc_m c_m over the
// explicit (non-default) concentration dependences, from which the
// assembly forms the column sums of the block without reading it back.
template <class CT>
__device__ __forceinline__ void jac_reaction(int qq, const StateScalars& s,
                                             CT c, CT g, CT h, double* D,
                                             double* Dq, double* DdT,
                                             double* Hq, double* Qc) {
  const double T = s.T, lnT = s.lnT, invT = s.invT;
  const int f = __ldg(jq_flags + qq);
  const int kind = f & RX_KIND_MASK;
  const int form = (f >> RX_FORM_SHIFT) & 3;
  const int s0 = __ldg(jq_slot0 + qq), s2 = __ldg(jq_slot0 + qq + 1);
  const int s1 = s0 + __ldg(jq_nr + qq);
  const double p0 = __ldg(&jq_rate[0][qq]), p1 = __ldg(&jq_rate[1][qq]),
               p2 = __ldg(&jq_rate[2][qq]);
  double m = 1.0, mt = 0.0;
  if (kind != RX_ELEMENTARY) {
    const double d = __ldg(jq_defeff + qq);
    m = d == 0.0 ? 0.0 : (d == 1.0 ? s.ctot : d * s.ctot);
    const int t1 = __ldg(jq_tb0 + qq + 1);
    for (int t = __ldg(jq_tb0 + qq); t < t1; ++t) {
      const double v = __ldg(jq_tbde + t) * c[__ldg(jq_tbidx + t)];
      m += v;
      mt += v;
    }
  }
  double kf, x = 0.0, dlnkf, dkfdM = 0.0;
  bool exp_form = false;
  if (kind == RX_FALLOFF) {
    const int sl = __ldg(jq_fo + qq);
    const int lform = __ldg(jf_lowform + sl);
    const double l0 = __ldg(&jf_low[0][sl]), l1 = __ldg(&jf_low[1][sl]),
                 l2 = __ldg(&jf_low[2][sl]);
    double xh, xl;
    const double k_hi = arrhenius(form, p0, p1, p2, T, lnT, invT, xh);
    const double k_lo = arrhenius(lform, l0, l1, l2, T, lnT, invT, xl);
    const double dxh = darr_dT(form, p1, p2, invT);
    const double dxl = darr_dT(lform, l1, l2, invT);
    const bool troe = (f & RX_TROE) != 0, troe_t2 = (f & RX_TROE_T2) != 0;
    const FalloffDeriv fd = falloff_deriv(
        troe, troe_t2, __ldg(&jf_troe[0][sl]), __ldg(&jf_troe[1][sl]),
        __ldg(&jf_troe[2][sl]), __ldg(&jf_troe[3][sl]),
        __ldg(&jf_troe[4][sl]), T, invT, m, k_hi, k_lo, dxh, dxl);
    kf = fd.kf;
    dlnkf = fd.dlnkf;
    dkfdM = fd.dkfdM;
  } else {
    const double ek = arrhenius(form, p0, p1, p2, T, lnT, invT, x);
    exp_form = form == FORM_EXP;
    dlnkf = darr_dT(form, p1, p2, invT);
    if (kind == RX_THREE_BODY) {
      kf = ek * m;
      dkfdM = ek;
    } else {
      kf = ek;
    }
  }
  // side products and the log K sums (signed stoichiometry per slot)
  double pf = 1.0, pv = 1.0, sg = 0.0, shh = 0.0;
  for (int a = s0; a < s2; ++a) {
    const int k = __ldg(jq_sp + a);
    const double cv = c[k];
    const double e = __ldg(jq_e + a), nu = __ldg(jq_nu + a);
    if (a < s1)
      pf *= ipow_or_pow(cv, e);
    else
      pv *= ipow_or_pow(cv, e);
    sg = fma(nu, g[k], sg);
    shh = fma(nu, h[k], shh);
  }
  double kr = 0.0, dlnkr = 0.0, dkrdM = 0.0;
  if (f & RX_REVERSIBLE) {
    const double dnu = __ldg(jq_dnu + qq);
    double lk = sg;
    if (dnu != 0.0) lk -= dnu * s.c0;
    const double dlk = (dnu - shh) * invT;
    if (exp_form) {
      const double ekr = PEXP(x + lk);
      kr = kind == RX_THREE_BODY ? ekr * m : ekr;
      dkrdM = kind == RX_THREE_BODY ? ekr : 0.0;
    } else {
      const double eK = PEXP(lk);
      kr = kf * eK;
      dkrdM = dkfdM * eK;
    }
    dlnkr = dlnkf + dlk;
  } else {
    pv = 0.0;
  }
  Dq[qq] = kf * pf - kr * pv;
  DdT[qq] = kf * dlnkf * pf - kr * dlnkr * pv;
  const double dqdm = dkfdM * pf - dkrdM * pv;
  D[NSLOT + qq] = dqdm;
  Hq[qq] = shh;
  double qc = dqdm * mt;
  // dq/dc per slot: kf d(prod c^e)/dc (reactants), -kr d(prod c^nu'')/dc
  for (int a = s0; a < s2; ++a) {
    const bool rside = a < s1;
    const int b0 = rside ? s0 : s1, b1 = rside ? s1 : s2;
    double others = 1.0, ea = 1.0;
    for (int b = b0; b < b1; ++b) {
      const double e = __ldg(jq_e + b);
      if (b == a)
        ea = e;
      else
        others *= ipow_or_pow(c[__ldg(jq_sp + b)], e);
    }
    const double cm = c[__ldg(jq_sp + a)];
    double d;
    if (ea == 1.0)
      d = 1.0;
    else if (ea == 2.0)
      d = 2.0 * cm;
    else
      d = ea * pow(cm, ea - 1.0);
    const double da = rside ? kf * (d * others) : -kr * (d * others);
    D[a] = da;
    qc = fma(da, cm, qc);
  }
  Qc[qq] = qc;
}

}  // namespace pyro

// A state is handled by a group of JGROUP threads: 8 or 16 lanes of a warp
// for small mechanisms (a warp then serves 4 or 2 states, so its species
// and reaction rounds keep most lanes busy), one warp, or two for large
// mechanisms (the per-state shared memory then holds an SM to half the
// states but still 16 warps, which the FP64 pipe needs to stay busy).
// Group-wide sums reduce within the group's lanes (xor shuffles inside the
// aligned group) or, for two warps, within each warp and then across them
// through shared memory in a fixed order, behind a named barrier.
namespace pyro {

__device__ __forceinline__ void group_sync(int gid) {
#if JGROUP <= 32
  (void)gid;
  __syncwarp();
#else
  asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(JGROUP) : "memory");
#endif
}

__device__ __forceinline__ double group_sum(double v, int gid, int t,
                                            double* red) {
#if JGROUP < 32
  (void)gid;
  (void)t;
  (void)red;
#pragma unroll
  for (int o = JGROUP / 2; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
#else
  v = warp_sum(v);
#endif
#if JGROUP == 32
  (void)gid;
  (void)t;
  (void)red;
  return v;
#elif JGROUP > 32
  if ((t & 31) == 0) red[t >> 5] = v;
  group_sync(gid);
  double r = red[0];
#pragma unroll
  for (int h = 1; h < JGROUP / 32; ++h) r += red[h];
  group_sync(gid);  // before the slots are written again
  return r;
#endif
}

}  // namespace pyro

// doubles of shared memory per group (JW_DOUBLES, from the tables):
//   c, h, g, cp, w, jt, a, u, shj [NS each]; q, dq/dT, Hq, Qc [NR each];
//   D = dq/dc per slot [NSLOT], dq/dM per reaction [NR], one zero.
// With F non-null the kernel also writes the source f = (dT/dt, dY/dt)
// [S+1][ldf] from the rates it forms anyway (the primal jacfwd returns with
// the tangents, flamelets/equations.py:124-129): one pass for both.
__global__ void __launch_bounds__(JGROUPS * JGROUP)
    k_reactor_jacobian(const double* __restrict__ Pp, int64_t p_inc,
                       const double* __restrict__ Tp, int64_t t_inc,
                       const double* __restrict__ Y, int64_t ldy,
                       double* __restrict__ J, int64_t ldj,
                       double* __restrict__ F, int64_t ldf, int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  const int t = threadIdx.x % JGROUP, gid = threadIdx.x / JGROUP;
  __shared__ double s_red[JGROUPS][JGROUP >= 32 ? JGROUP / 32 : 1];
  double* red = s_red[gid];
  double* sc = smem + (size_t)gid * JW_DOUBLES;
  double* sh = sc + NS;
  double* sg = sh + NS;   // g/RT, later the row constants B_k
  double* scp = sg + NS;
  double* sw = scp + NS;
  double* sjt = sw + NS;  // later the column-0 values
  double* sa = sjt + NS;
  double* su = sa + NS;
  double* shj = su + NS;
  double* Dq = shj + NS;
  double* DdT = Dq + NR;
  double* Hq = DdT + NR;
  double* Qc = Hq + NR;
  double* D = Qc + NR;  // [NSLOT] dq/dc, [NR] dq/dM, [1] zero
  using LC = pyro::LocalCols;
  const LC c{sc}, g{sg}, h{sh};
  constexpr int NC = NS + 1;
  if (t == 0) D[JD_ZERO] = 0.0;
  // the groups of one warp (sub-warp groups) step through states together,
  // so every lane reaches the warp-wide shuffles; a group past the last
  // state works on a copy of it and stores nothing
  constexpr int GPW = JGROUP < 32 ? 32 / JGROUP : 1;
  for (int64_t i0 = (int64_t)blockIdx.x * JGROUPS + gid - gid % GPW; i0 < n;
       i0 += (int64_t)gridDim.x * JGROUPS) {
    const bool live = i0 + gid % GPW < n;
    const int64_t i = live ? i0 + gid % GPW : n - 1;
    double* Ji = J + i * ldj;
    const double T = pyro_ld(Tp, t_inc, i);
    const double P = pyro_ld(Pp, p_inc, i);
    const double lnT = log(T), invT = 1.0 / T;
    // species thermo, sigma, cp, dcp/dT (threads over species)
    double sig = 0.0, cpp = 0.0, dcpp = 0.0;
    for (int k = t; k < NS; k += JGROUP) {
      const double* nk = &jg_nasa[k][0];
      const bool up = T > __ldg(nk);
      const double* a = nk + (up ? 1 : 8);
      double q[7];
#pragma unroll
      for (int t = 0; t < 7; ++t) q[t] = __ldg(a + t);
      const double cpk =
          fma(T, fma(T, fma(T, fma(T, q[4], q[3]), q[2]), q[1]), q[0]);
      const double hk =
          fma(T, fma(T, fma(T, fma(T, q[4] * 0.2, q[3] * 0.25),
                            q[2] * (1.0 / 3.0)),
                    q[1] * 0.5),
              q[0]) +
          q[5] * invT;
      const double gk =
          fma(q[0], 1.0 - lnT, fma(q[5], invT, -q[6])) -
          T * fma(T, fma(T, fma(T, q[4] * (1.0 / 20.0), q[3] * (1.0 / 12.0)),
                         q[2] * (1.0 / 6.0)),
                  q[1] * 0.5);
      const double dcpk =
          fma(T, fma(T, 4.0 * q[4], 3.0 * q[3]), 2.0 * q[2]) * T + q[1];
      const double wk = __ldg(Y + (int64_t)k * ldy + i) * __ldg(jg_invmw + k);
      scp[k] = cpk;
      sh[k] = hk;
      sg[k] = gk;
      sig += wk;
      cpp = fma(wk, cpk, cpp);
      dcpp = fma(wk, dcpk, dcpp);
    }
    const double sigma = pyro::group_sum(sig, gid, t, red);
    const double cpm = GAS_CONSTANT * pyro::group_sum(cpp, gid, t, red);
    const double dcpm = GAS_CONSTANT * pyro::group_sum(dcpp, gid, t, red);
    const double rho = P / (GAS_CONSTANT * T * sigma);
    double ct = 0.0;
    for (int k = t; k < NS; k += JGROUP) {
      const double v =
          __ldg(jg_invmw + k) * rho * __ldg(Y + (int64_t)k * ldy + i);
      sc[k] = v;
      ct += v;
    }
    pyro::StateScalars s;
    s.T = T;
    s.lnT = lnT;
    s.invT = invT;
    s.c0 = LOG_P0_OVER_R - lnT;
    s.ctot = pyro::group_sum(ct, gid, t, red);
    pyro::group_sync(gid);
    // per reaction: lane blocks of one kind per warp and round (the
    // generated map jq_lane_rx; -1 for an idle lane)
#pragma unroll 1
    for (int rd = 0; rd < JQ_ROUNDS; ++rd) {
      const int qq = __ldg(jq_lane_rx + rd * JGROUP + t);
      if (qq >= 0) pyro::jac_reaction(qq, s, c, g, h, D, Dq, DdT, Hq, Qc);
    }
    pyro::group_sync(gid);
    const double RT = GAS_CONSTANT * T;
    const double inv_sig = 1.0 / sigma;
    // the sums run over parts of each species' slot list of nearly equal
    // length (generated: jp_*), one per thread and round; a species' other
    // parts leave their partial sums in the dead q vector for its owner
    double pw[JP_ROUNDS], pjt[JP_ROUNDS], pa[JP_ROUNDS], pu[JP_ROUNDS],
        phj[JP_ROUNDS];
#pragma unroll
    for (int rd = 0; rd < JP_ROUNDS; ++rd) {
      const int e = rd * JGROUP + t;
      double w = 0.0, jt = 0.0, a = 0.0, u = 0.0, hj = 0.0;
      if (__ldg(jp_sp + e) >= 0) {
        const int t1 = __ldg(jp_s1 + e);
        for (int t = __ldg(jp_s0 + e); t < t1; ++t) {
          const int sl = __ldg(jg_si_slot + t);
          const int qq = __ldg(jq_slot_rx + sl);
          const double nu = __ldg(jq_nu + sl);
          w = fma(nu, Dq[qq], w);
          jt = fma(nu, DdT[qq], jt);
          a = fma(__ldg(jq_slot_anu + sl), D[NSLOT + qq], a);
          u = fma(nu, Qc[qq], u);
          hj = fma(Hq[qq], D[sl], hj);
        }
        const int e1 = __ldg(jp_t1 + e);
        for (int t = __ldg(jp_t0 + e); t < e1; ++t) {
          const int qq = __ldg(jg_st_q + t);
          hj = fma(Hq[qq] * __ldg(jg_st_de + t), D[NSLOT + qq], hj);
        }
      }
      pw[rd] = w;
      pjt[rd] = jt;
      pa[rd] = a;
      pu[rd] = u;
      phj[rd] = hj;
    }
    pyro::group_sync(gid);  // every thread is done with Dq
    double* px = Dq;
#pragma unroll
    for (int rd = 0; rd < JP_ROUNDS; ++rd) {
      const int sl = __ldg(jp_slot + rd * JGROUP + t);
      if (sl >= 0) {
        px[5 * sl] = pw[rd];
        px[5 * sl + 1] = pjt[rd];
        px[5 * sl + 2] = pa[rd];
        px[5 * sl + 3] = pu[rd];
        px[5 * sl + 4] = phj[rd];
      }
    }
    pyro::group_sync(gid);
    // per species k (its owner thread): w_k, dw_k/dT|c, the rank-1
    // third-body vector a_k, u_k = sum_m dw_k/dc_m c_m and the column sum
    // shj_k = RT sum_j h_j dw_j/dc_k; then the row constants of the
    // assembly
    double pQ = 0.0, pHA = 0.0, pHU = 0.0, pdQ = 0.0;
#pragma unroll
    for (int rd = 0; rd < JP_ROUNDS; ++rd) {
      const int e = rd * JGROUP + t;
      const int k = __ldg(jp_sp + e);
      if (k < 0 || __ldg(jp_slot + e) >= 0) continue;
      double w = pw[rd], jt = pjt[rd], a = pa[rd], u = pu[rd], hj = phj[rd];
      const int x1 = __ldg(jp_x0 + k + 1);
      for (int x = __ldg(jp_x0 + k); x < x1; ++x) {
        const double* q = px + 5 * __ldg(jp_xslot + x);
        w += q[0];
        jt += q[1];
        a += q[2];
        u += q[3];
        hj += q[4];
      }
      u = fma(a, s.ctot, u);
      sw[k] = w;
      sa[k] = a;
      su[k] = u;
      shj[k] = RT * hj;
      const double Hk = RT * sh[k];
      pQ = fma(Hk, w, pQ);
      pHA = fma(Hk, a, pHA);
      pHU = fma(Hk, u, pHU);
      // dQ/dT = sum_k (R cp_k w_k + H_k (dw_k/dT|c - u_k / T))
      pdQ += GAS_CONSTANT * scp[k] * w + Hk * (jt - u * invT);
      const double wk_rho = __ldg(jg_mw + k) / rho;
      sg[k] = wk_rho * fma(a, rho, (w - u) * inv_sig);  // B_k
      sjt[k] = wk_rho * (jt - u * invT + w * invT);     // column 0
    }
    const double Q = pyro::group_sum(pQ, gid, t, red);
    const double HA = pyro::group_sum(pHA, gid, t, red);
    const double HU = pyro::group_sum(pHU, gid, t, red);
    const double dQdT = pyro::group_sum(pdQ, gid, t, red);
    const double rcp = rho * cpm;
    const double inv_rcp = 1.0 / rcp;
    const double qr2 = Q * inv_rcp * inv_rcp;
    if (F != nullptr) {
      // dT/dt = -Q / (rho cp), dY_k/dt = W_k w_k / rho (the thread that
      // formed w_k stores it)
      if (live && t == 0) F[i] = -Q * inv_rcp;
      for (int k = t; live && k < NS; k += JGROUP)
        F[(int64_t)(k + 1) * ldf + i] = __ldg(jg_mw + k) * sw[k] / rho;
    }
    pyro::group_sync(gid);
    // rows 1..S, columns 1..S: d(dY_k/dt)/dY_m = W_k/rho ((Jc + a_k) rho
    //   / W_m + (w_k - u_k) / (sigma W_m)) = (W_k Jc_km + B_k) / W_m with
    // Jc = dw/dc.  Elements of dw/dc without contributions are B_k / W_m;
    // the others are summed by the lane that owns them (its run of the
    // update list) and stored once, transformed, with no read-back.
    for (int it = 0; it < JZ_ITERS; ++it) {
      const int off = __ldg(jz_off + it * JGROUP + t);
      if (live && off != 0xFFFF) {
        const int k = off / NC - 1, m = off - (k + 1) * NC - 1;
        Ji[off] = __ldg(jg_invmw + m) * sg[k];
      }
    }
    {
      int cur = -1;
      double acc = 0.0;
      for (int it = 0; it < JU_ITERS; ++it) {
        const int e = it * JGROUP + t;
        const int off = __ldg(ju_off + e);
        const double cf = __ldg(ju_coef + e);
        const double dv = D[__ldg(ju_src + e)];
        if (off != cur) {
          if (live && cur >= 0 && cur != 0xFFFF) {
            const int k = cur / NC - 1, m = cur - (k + 1) * NC - 1;
            Ji[cur] = __ldg(jg_invmw + m) * fma(__ldg(jg_mw + k), acc, sg[k]);
          }
          cur = off;
          acc = 0.0;
        }
        acc = fma(cf, dv, acc);
      }
      if (live && cur >= 0 && cur != 0xFFFF) {
        const int k = cur / NC - 1, m = cur - (k + 1) * NC - 1;
        Ji[cur] = __ldg(jg_invmw + m) * fma(__ldg(jg_mw + k), acc, sg[k]);
      }
    }
    // row 0: d(dT/dt)/dx
    for (int col = t; col < NC; col += JGROUP) {
      double v;
      if (col == 0) {
        v = -dQdT * inv_rcp + qr2 * (-rcp * invT + rho * dcpm);
      } else {
        const int jj = col - 1;
        const double iw = __ldg(jg_invmw + jj);
        const double dQdY = rho * iw * (shj[jj] + HA) - HU * inv_sig * iw;
        const double drcp =
            -rcp * inv_sig * iw + rho * GAS_CONSTANT * scp[jj] * iw;
        v = -dQdY * inv_rcp + qr2 * drcp;
      }
      if (live) Ji[col] = v;
    }
    // column 0 of rows 1..S
    for (int k = t; live && k < NS; k += JGROUP)
      Ji[(int64_t)(k + 1) * NC] = sjt[k];
    pyro::group_sync(gid);
  }
}

// Source values f = (dT/dt, dY/dt) [S+1][ldf] (table-driven, one thread
// per state).
__global__ void __launch_bounds__(BLOCK)
    k_reactor_source(const double* __restrict__ Pp, int64_t p_inc,
                     const double* __restrict__ Tp, int64_t t_inc,
                     const double* __restrict__ Y, int64_t ldy,
                     double* __restrict__ F, int64_t ldf, int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  const pyro::Cols c = pyro::col(smem, 0), g = pyro::col(smem, 1),
                   w = pyro::col(smem, 2);
  PYRO_LOOP(i) {
    const double T = pyro_ld(Tp, t_inc, i);
    const double lnT = log(T), invT = 1.0 / T;
    double sigma = 0.0, cpp = 0.0;
    for (int k = 0; k < NS; ++k) {
      const double wk = __ldg(Y + (int64_t)k * ldy + i) * k_inv_mw[k];
      sigma += wk;
      const pyro::Nasa a(k, T > k_tmid[k]);
      cpp = fma(wk,
                fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]),
                cpp);
    }
    const double rho = pyro_ld(Pp, p_inc, i) / (GAS_CONSTANT * T * sigma);
    const pyro::StateScalars s = pyro::state_from_mass(T, rho, Y, ldy, i, c);
    pyro::production_rates(s, c, g, w);
    double q = 0.0;
    for (int k = 0; k < NS; ++k) {
      const pyro::Nasa a(k, T > k_tmid[k]);
      const double hrt =
          fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                            a[2] * (1.0 / 3.0)),
                    a[1] * 0.5),
              a[0]) +
          a[5] * invT;
      q = fma(GAS_CONSTANT * T * hrt, w[k], q);
      F[(int64_t)(k + 1) * ldf + i] = k_mw[k] * w[k] / rho;
    }
    F[i] = -q / (rho * GAS_CONSTANT * cpp);
  }
}

// df/dp at fixed (T, Y), F [S+1][ldf], for f = (dT/dt, W w / rho): the
// concentrations and [M] scale with p (rho = p / (R T sigma)), so
// dq/d ln p = rf (n_f + m) - rr (n_r + m) per reaction, n_f / n_r the sums
// of its forward orders / product coefficients and m = d ln kf / d ln [M]
// (the homogeneity of mass-action rates), then
//   d(W_k w_k / rho)/dp = (W_k / rho) (dw_k / d ln p - w_k) / p,
//   d(dT/dt)/dp = -(sum_k H_k dw_k / d ln p) / (rho cp p) - (dT/dt) / p.
// The forward-mode pressure derivative the reference takes with jacfwd
// (FlameletEquations.source_gradient_wrt_pressure, equations.py:130-134).
#ifndef DPBLOCK
#define DPBLOCK 64
#endif

__global__ void __launch_bounds__(DPBLOCK)
    k_reactor_source_dp(const double* __restrict__ Pp, int64_t p_inc,
                        const double* __restrict__ Tp, int64_t t_inc,
                        const double* __restrict__ Y, int64_t ldy,
                        double* __restrict__ F, int64_t ldf, int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  using DC = pyro::ColsT<DPBLOCK>;
  double* col0 = smem + threadIdx.x;
  const DC c{col0}, g{col0 + NS * DPBLOCK}, w{col0 + 2 * NS * DPBLOCK},
      dw{col0 + 3 * NS * DPBLOCK};
  for (int64_t i = (int64_t)blockIdx.x * DPBLOCK + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * DPBLOCK) {
    const double T = pyro_ld(Tp, t_inc, i);
    const double lnT = log(T), invT = 1.0 / T;
    double sigma = 0.0, cpp = 0.0;
    for (int k = 0; k < NS; ++k) {
      const double wk = __ldg(Y + (int64_t)k * ldy + i) * k_inv_mw[k];
      sigma += wk;
      const pyro::Nasa a(k, T > k_tmid[k]);
      cpp = fma(wk,
                fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]),
                cpp);
    }
    const double P = pyro_ld(Pp, p_inc, i);
    const double rho = P / (GAS_CONSTANT * T * sigma);
    const pyro::StateScalars s = pyro::state_from_mass(T, rho, Y, ldy, i, c);
    pyro::gibbs_all(s.T, s.lnT, s.invT, g);
    for (int k = 0; k < NS; ++k) {
      w[k] = 0.0;
      dw[k] = 0.0;
    }
    for (int j = 0; j < NR; ++j) {
      double kf, rf, rr, mlog;
      pyro::reaction_rates(j, s.T, s.lnT, s.invT, s.c0, s.ctot, c, g, true,
                           kf, rf, rr, &mlog);
      const int fl = k_rx_flags[j];
      const int nr = k_rx_nr[j], np = k_rx_np[j];
      const bool frac = (fl & RX_FRACTIONAL) != 0;
      const int fr = k_rx_frac[j];
      double nf = 0.0, nb = 0.0;
      for (int a = 0; a < MAXSIDE; ++a) {
        if (a < nr)
          nf += frac ? k_frac[fr][2 * MAXSIDE + a] : (double)k_rx_ord[j][a];
        if (a < np)
          nb += frac ? k_frac[fr][MAXSIDE + a]
                     : (double)k_rx_nu[j][MAXSIDE + a];
      }
      pyro::scatter_net(j, rf - rr, w);
      pyro::scatter_net(j, rf * (nf + mlog) - rr * (nb + mlog), dw);
    }
    double q = 0.0, dq = 0.0;
    const double invP = 1.0 / P;
    for (int k = 0; k < NS; ++k) {
      const pyro::Nasa a(k, T > k_tmid[k]);
      const double hrt =
          fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                            a[2] * (1.0 / 3.0)),
                    a[1] * 0.5),
              a[0]) +
          a[5] * invT;
      const double H = GAS_CONSTANT * T * hrt;
      q = fma(H, w[k], q);
      dq = fma(H, dw[k], dq);
      F[(int64_t)(k + 1) * ldf + i] = k_mw[k] / rho * (dw[k] - w[k]) * invP;
    }
    const double rcp = rho * GAS_CONSTANT * cpp;
    F[i] = (-dq / rcp + q / rcp) * invP;
  }
}

// Vector-Jacobian product v^T df/dx for x = (T, Y) and df/dp, with v
// [S+1][ldv]; outputs gT[n], gY[S][ldg], gp[n] (gp may be NULL).
#ifndef VBLOCK
#define VBLOCK 32
#endif

__global__ void __launch_bounds__(VBLOCK)
    k_reactor_vjp(const double* __restrict__ Pp, int64_t p_inc,
                  const double* __restrict__ Tp, int64_t t_inc,
                  const double* __restrict__ Y, int64_t ldy,
                  const double* __restrict__ V, int64_t ldv,
                  double* __restrict__ gT, double* __restrict__ gY,
                  int64_t ldg, double* __restrict__ gp, int64_t n) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
  using VC = pyro::ColsT<VBLOCK>;
  double* col0 = smem + threadIdx.x;
  const VC c{col0}, g{col0 + NS * VBLOCK}, h{col0 + 2 * NS * VBLOCK},
      gc{col0 + 3 * NS * VBLOCK}, w{col0 + 4 * NS * VBLOCK};
  for (int64_t i = (int64_t)blockIdx.x * VBLOCK + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * VBLOCK) {
    const double T = pyro_ld(Tp, t_inc, i);
    const double P = pyro_ld(Pp, p_inc, i);
    const double lnT = log(T), invT = 1.0 / T;
    double sigma = 0.0, cpp = 0.0, dcpp = 0.0;
    for (int k = 0; k < NS; ++k) {
      const double wk = __ldg(Y + (int64_t)k * ldy + i) * k_inv_mw[k];
      const pyro::SpThermo th = pyro::species_thermo(k, T, lnT, invT);
      h[k] = th.h;
      g[k] = th.g;
      sigma += wk;
      cpp = fma(wk, th.cp, cpp);
      dcpp = fma(wk, th.dcp, dcpp);
      gc[k] = 0.0;
      w[k] = 0.0;
    }
    const double cpm = GAS_CONSTANT * cpp, dcpm = GAS_CONSTANT * dcpp;
    const double rho = P / (GAS_CONSTANT * T * sigma);
    double ct = 0.0;
    for (int k = 0; k < NS; ++k) {
      const double v = k_inv_mw[k] * rho * __ldg(Y + (int64_t)k * ldy + i);
      c[k] = v;
      ct += v;
    }
    pyro::StateScalars s;
    s.T = T;
    s.lnT = lnT;
    s.invT = invT;
    s.c0 = LOG_P0_OVER_R - lnT;
    s.ctot = ct;
    const double RT = GAS_CONSTANT * T;
    const double rcp = rho * cpm;
    const double v0 = __ldg(V + i);
    // lambda_k = v_k W_k / rho - v0 H_k / (rho cp)
    const double l1 = 1.0 / rho, l2 = -v0 * RT / rcp;
    double gTc = 0.0, A = 0.0;
    for (int r = 0; r < NR; ++r) {
      const pyro::RxnDeriv d = pyro::reaction_deriv(r, s, c, g, h);
      const int f = k_rx_flags[r];
      const int nr = k_rx_nr[r], np = k_rx_np[r];
      double mu = 0.0;
      for (int a = 0; a < MAXSIDE; ++a) {
        if (a < nr) {
          const int k = k_rx_sp[r][a];
          const double nu = pyro::slot_nu(r, a);
          const double lam =
              fma(__ldg(V + (int64_t)(k + 1) * ldv + i) * k_mw[k], l1,
                  l2 * h[k]);
          mu = fma(nu, lam, mu);
          w[k] = fma(nu, d.q, w[k]);
        }
        if (a < np) {
          const int k = k_rx_sp[r][MAXSIDE + a];
          const double nu = pyro::slot_nu(r, MAXSIDE + a);
          const double lam =
              fma(__ldg(V + (int64_t)(k + 1) * ldv + i) * k_mw[k], l1,
                  l2 * h[k]);
          mu = fma(nu, lam, mu);
          w[k] = fma(nu, d.q, w[k]);
        }
      }
      gTc = fma(mu, d.dqdT, gTc);
      const bool frac = (f & RX_FRACTIONAL) != 0;
      for (int a = 0; a < MAXSIDE; ++a) {
        if (a < nr) {
          const int k = k_rx_sp[r][a];
          gc[k] = fma(mu * d.kf, pyro::dprod(r, 0, a, nr, frac, c), gc[k]);
        }
        if (a < np) {
          const int k = k_rx_sp[r][MAXSIDE + a];
          gc[k] = fma(-mu * d.kr, pyro::dprod(r, 1, a, np, frac, c), gc[k]);
        }
      }
      if ((f & RX_KIND_MASK) != RX_ELEMENTARY) {
        const double md = mu * d.dqdM;
        A = fma(md, k_rx_defeff[r], A);
        for (int t = k_rx_tb[r]; t < k_rx_tb[r + 1]; ++t)
          gc[k_tb_idx[t]] = fma(md, k_tb_de[t], gc[k_tb_idx[t]]);
      }
    }
    double GC = 0.0, Q = 0.0, S1 = 0.0, S3 = 0.0;
    for (int k = 0; k < NS; ++k) {
      gc[k] += A;
      GC = fma(gc[k], c[k], GC);
      Q = fma(RT * h[k], w[k], Q);
      S1 = fma(__ldg(V + (int64_t)(k + 1) * ldv + i) * k_mw[k], w[k], S1);
    }
    for (int k = 0; k < NS; ++k) {
      const pyro::Nasa a(k, T > k_tmid[k]);
      const double cpr =
          fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
      S3 = fma(GAS_CONSTANT * cpr, w[k], S3);
    }
    const double inv_sig = 1.0 / sigma;
    const double qf = v0 * Q / (rcp * cpm);
    gT[i] = gTc - GC * invT + S1 * invT / rho - v0 * S3 / rcp +
            qf * (-cpm * invT + dcpm);
    for (int k = 0; k < NS; ++k) {
      const pyro::Nasa a(k, T > k_tmid[k]);
      const double cpr =
          fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
      const double iw = k_inv_mw[k];
      gY[(int64_t)k * ldg + i] =
          gc[k] * rho * iw + (S1 / rho - GC) * inv_sig * iw +
          qf * (-cpm * inv_sig * iw + GAS_CONSTANT * cpr * iw);
    }
    if (gp) gp[i] = (GC - S1 / rho + v0 * Q / rcp) / P;
  }
}
