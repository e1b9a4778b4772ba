// Hand-written adjoint of the per-cell NSW6 physics (nsw6_cell, the reference
// configuration), for both precisions of the step.
//
// One call recomputes the cell's forward values exactly as nsw6_cell does
// (same operations, same branches) and then runs the reverse sweep statement
// by statement, from the outputs' adjoints back to the inputs' and the seven
// parameters'.  Nothing is recorded: the values the sweep needs stay in the
// thread's registers (and its local memory), so the cost is arithmetic, where
// a recorded tape costs about 32 bytes of memory traffic per operation.
//
// R is the precision of the process rates, as in nsw6_cell: double for the
// FP64 step, float for the mixed-precision step (FP32 saturation values,
// rates, limiters, tendencies, fall speeds and effective radii; FP64 negative
// filter, budgets and temperature).  The sweep runs each part in the
// precision of its forward: the adjoints of the FP32 rates are FP32, those of
// the budgets FP64, and the input and parameter adjoints are accumulated in
// FP64.
//
// The derivative of every elementary operation is the one the recording
// adjoint (nsw6_ad.cuh, RVar) takes: quotients, products, sums and fused
// multiply-adds by their partials; min / max / select and every branch follow
// the values; exp, log and pow by their closed forms at the computed values.
// Both adjoints are compared on every cell by the GPU tests (FP64).
//
// Parameters (nsw6_params order): 0 beta_saut, 1 qicrt_saut, 2 Cr, 3 Cs, 4 Cg,
// 5 ice_nuc, 6 kk_aut; they enter through the constants folded from them
// (consts_with_params, nsw6_column_step.cuh).
#pragma once

#include "nsw6_cell.cuh"
#include "nsw6_common.cuh"
#include "nsw6_fastmath.cuh"

namespace nsw6 {

// Adjoints of the cell outputs (seeds); q[0] is passed through and unused.
struct CellBar {
  double rhog, rhoge, tem;
  double rhogq[6];
  double q[6];
  double Vtr, Vts, Vtg;
  double rceff, rceff_cld, rctop, tctop;
};

// Adjoints of the cell inputs.
struct CellInBar {
  double rhog, tem, gsgam2, q0;
  double rhogq[6];
};

// d(min(a, b)): the adjoint g goes to the operand min chose, as dmin.
template <class T>
__device__ __forceinline__ void bmin(T a, T b, T g, T& ba, T& bb) {
  if (b < a) bb += g;
  else ba += g;
}
template <class T>
__device__ __forceinline__ void bmax(T a, T b, T g, T& ba, T& bb) {
  if (a < b) bb += g;
  else ba += g;
}
// d(max(a, 0)) and d(max(a, c)) for a constant c > 0: the comparisons of
// bmax with the integer-pipe forms of nsw6_cell.cuh
template <class T>
__device__ __forceinline__ void bmaxz(T a, T g, T& ba, T& bb) {
  if (lt_z(a)) bb += g;
  else ba += g;
}
template <class T>
__device__ __forceinline__ void bmaxc(T a, T c, T g, T& ba, T& bb) {
  if (lt_c(a, c)) bb += g;
  else ba += g;
}
// d sqrt(x) / dx from s = sqrt(x)
__device__ __forceinline__ double bsqrt(double s) { return s > 0.0 ? 0.5 / s : 0.0; }
__device__ __forceinline__ float bsqrt(float s) { return s > 0.0f ? 0.5f / s : 0.0f; }

// How a call treats the forward's costly values (quotients, square roots,
// exp / log / pow; CELL_CK_SLOTS of them, each computed at most once):
//   CA_FULL  computes them, then runs the reverse sweep;
//   CA_SAVE  computes them and stores them to the cell's checkpoint, writes
//            the cell outputs (those of nsw6_cell) and returns;
//   CA_LOAD  reads them from the checkpoint instead, then runs the reverse.
// The stored values are the computed ones, so every branch takes the same way
// in all three.
enum CellAdjMode { CA_FULL = 0, CA_SAVE = 1, CA_LOAD = 2 };
constexpr int CELL_CK_SLOTS = 49;
// The checkpoint of cell c: slot s at element c + s * stride of the buffer p
// viewed as an array of the rate precision R (the buffer holds CELL_CK_SLOTS
// doubles per cell).  The mixed-precision step's FP32 slots use its first
// half (slot 1, the density, is FP32 there); its FP64 slots (0: 1 / rhog,
// 48: the temperature) sit as doubles at rows CK_MIXED_D and CK_MIXED_D + 2 of
// the second.
struct CellCk {
  double* p;
  size_t stride, c;
};
constexpr int CK_MIXED_D = (CELL_CK_SLOTS + 1) / 2;
// Where slot s (of type T) of the cell lives.
template <class R, class T>
__device__ __forceinline__ T* ck_ptr(const CellCk& ck, int s) {
  if constexpr (sizeof(T) != sizeof(R))
    return reinterpret_cast<T*>(ck.p) + ck.c + (size_t)(CK_MIXED_D + (s == 0 ? 0 : s == 1 ? 1 : 2)) * ck.stride;
  else
    return reinterpret_cast<T*>(ck.p) + ck.c + (size_t)s * ck.stride;
}
template <int MODE, class R, class T>
__device__ __forceinline__ T ck_keep(const CellCk& ck, int s, T v) {
  if constexpr (MODE == CA_SAVE) *ck_ptr<R, T>(ck, s) = v;
  return v;
}
// The value of expr (of type T; not evaluated under CA_LOAD) at slot s.
#define NSW6_CK(T, s, expr) ((MODE == CA_LOAD) ? *ck_ptr<R, T>(ck, (s)) : ck_keep<MODE, R, T>(ck, (s), (T)(expr)))

// R = double with FastMath (the FP64 step) or R = float with FloatMath (the
// mixed-precision step).
template <int MODE = CA_FULL, class R = double, class M = FastMath>
__device__ __forceinline__ void nsw6_cell_adjoint(const ConstsT<R>& C, const M& mth, double dt, double rdt,
                                                  const CellIn& in, const CellBar& ob, CellInBar& ib, double* pb,
                                                  CellCk ck = {nullptr, 0, 0}, CellOut* out = nullptr) {
  using D = double;
  constexpr bool kMixed = sizeof(R) == sizeof(float);
  const R Z = R(0.0), ONE = R(1.0);
  const R dtR = R(dt), rdtR = R(rdt);
  // ==================================================================== forward
  // ---- negative_filter, mod_mp_nsw6.cpp:1770-1831 (FP64)
  D rq[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] = in.rhogq[n];
  bool clip[6] = {false, false, false, false, false, false};
  D diffq = 0.0;
#pragma unroll
  for (int n = 2; n <= 5; ++n) {
    diffq += rq[n];
    clip[n] = lt_z(rq[n]);
    rq[n] = clip[n] ? 0.0 : rq[n];
  }
#pragma unroll
  for (int n = 2; n <= 5; ++n) diffq -= rq[n];
  rq[0] += diffq;
  D d2 = rq[0];
  clip[0] = lt_z(rq[0]);
  rq[0] = clip[0] ? 0.0 : rq[0];
  d2 -= rq[0];
  const D omd = 1.0 - d2;
  const D rhog = in.rhog * omd;
  const D rrhog = NSW6_CK(D, 0, 1.0 / rhog);
  D qn[6];
  qn[0] = in.q0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qn[n] = kMixed ? rq[n] * rrhog : div_rn(rq[n], rhog, rrhog);
  const D temp = in.tem;
  const D trh = temp * rhog;
  D dens, rhoge0, cv = CVDRY, pq = 0.0, dp = 0.0;
  R pre, densR, pqR = Z, dpR = Z;
  if constexpr (kMixed) {
    // as nsw6_cell: cv = CVdry (every CVW is CVdry), density and pressure in FP32
    rhoge0 = trh * CVDRY;
    densR = NSW6_CK(R, 1, R(rhog) / R(in.gsgam2));
    dens = D(densR);
    R qdR = ONE;
#pragma unroll
    for (int n = 1; n <= 5; ++n) qdR = qdR - R(qn[n]);
    pqR = qdR * R(RDRY) + R(qn[0]) * R(RVAP);
    dpR = densR * pqR;
    pre = dpR * R(temp);
  } else {
    dens = NSW6_CK(D, 1, rhog / in.gsgam2);
    D qd = 1.0;
#pragma unroll
    for (int n = 1; n <= 5; ++n) qd = qd - qn[n];
    cv = qd * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cv = cv + qn[n] * CVDRY;
    rhoge0 = trh * cv;
    pq = qd * RDRY + qn[0] * RVAP;
    dp = dens * pq;
    pre = R(dp * temp);
    densR = R(dens);
  }

  // ---- psat / qsat (rate precision from here to the tendencies)
  const R tempR = R(temp);
  const R tmx = maxc(tempR, R(TEM_MIN));
  const R rtem = NSW6_CK(R, 2, ONE / tmx);
  const R al = C.LovR_liq * (C.RTEM00 - rtem);
  const R ai = C.LovR_ice * (C.RTEM00 - rtem);
  const R el = NSW6_CK(R, 3, mth.exp(al)), ei = NSW6_CK(R, 4, mth.exp(ai));
  const R psatl = R(PSAT0) * el;
  const R psati = R(PSAT0) * ei;
  const R drv = densR * R(RVAP);
  const R drt = drv * tempR;
  const R rdrt = NSW6_CK(R, 5, ONE / drt);
  const R qsatl = psatl * rdrt;
  const R qsati = psati * rdrt;

  // ---- TagBigLoop
  const R qv = maxz(R(qn[0])), qc = maxz(R(qn[1])), qr = maxz(R(qn[2]));
  const R qi = maxz(R(qn[3])), qs = maxz(R(qn[4])), qg = maxz(R(qn[5]));
  const R sld = maxc(qsatl, R(EPS)), sid = maxc(qsati, R(EPS));
  const R Sliq = NSW6_CK(R, 6, qv / sld);
  const R Sice = NSW6_CK(R, 7, qv / sid);
  const R Rdens = NSW6_CK(R, 8, ONE / densR);
  const R rfa = R(DENS00) * Rdens;
  const R rho_fact = NSW6_CK(R, 9, sqrtR(rfa));
  const R temc = tempR - R(TEM00);
  const bool warm = !lt_z(temc);
  const bool d1 = ge_c(qr, R(1.0E-4));
  const bool d2b = le_c(qr, R(1.0E-4)) && le_c(qs, R(1.0E-4));
  const bool sps = ge_c(Sice, ONE);
  const R dqv_dt = per_dt(qv, dtR, rdtR), dqc_dt = per_dt(qc, dtR, rdtR), dqr_dt = per_dt(qr, dtR, rdtR);
  const R dqi_dt = per_dt(qi, dtR, rdtR), dqs_dt = per_dt(qs, dtR, rdtR), dqg_dt = per_dt(qg, dtR, rdtR);

  // rain slope parameter
  const bool rain = ge_c(qr, R(1.0E-12));
  R r_a = Z, r_b = Z;   // dens qr, (dens qr) K_rlmdr
  R r_s1 = Z;           // sqrt(r_b)
  R RLMDr = Z, RLMDr_dr = Z, RLMDr_2 = Z, RLMDr_3 = Z, RLMDr_1br = Z, RLMDr_2br = Z, RLMDr_3br = Z, RLMDr_7 = Z;
  R RLMDr_3dr = Z, RLMDr_5dr = Z, RLMDr_6dr = Z;
  if (rain) {
    r_a = densR * qr;
    r_b = r_a * C.K_rlmdr;
    r_s1 = NSW6_CK(R, 10, sqrtR(r_b));
    RLMDr = NSW6_CK(R, 11, sqrtR(r_s1));
    RLMDr_dr = NSW6_CK(R, 12, sqrtR(RLMDr));
    RLMDr_2 = RLMDr * RLMDr;
    RLMDr_3 = RLMDr_2 * RLMDr;
    RLMDr_1br = RLMDr_2 * RLMDr_2;
    RLMDr_2br = RLMDr_1br * RLMDr;
    RLMDr_3br = RLMDr_3 * RLMDr_3;
    RLMDr_7 = RLMDr_3br * RLMDr;
    RLMDr_3dr = RLMDr_3 * RLMDr_dr;
    RLMDr_5dr = RLMDr_2br * RLMDr_dr;
    RLMDr_6dr = RLMDr_3br * RLMDr_dr;
  }

  // Roh and Satoh (2014) snow moments
  const R xs_a = densR * qs;
  const R Xs2 = xs_a * C.rAs;
  const bool snow = ge_c(Xs2, R(1.0E-12));
  R mom[7] = {Z, Z, Z, Z, Z, Z, Z};
  R mlb[7] = {Z, Z, Z, Z, Z, Z, Z};   // b of each moment (d mom / d logX = mom b)
  R RMOMs_Vt = Z, logX = Z;
  R tems = Z;
  bool tems_sel = false;   // tems = temc (else the constant -0.1)
  if (snow) {
    tems_sel = lt_negc(temc, R(-0.1));   // dmin(-0.1, temc) is temc
    tems = tems_sel ? temc : R(-0.1);
    logX = NSW6_CK(R, 13, mth.log(Xs2));
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const R* a = C.roh_a + 4 * i;
      const R* b = C.roh_b + 4 * i;
      const R la = fmaR(fmaR(fmaR(a[3], tems, a[2]), tems, a[1]), tems, a[0]);
      const R lb = fmaR(fmaR(fmaR(b[3], tems, b[2]), tems, b[1]), tems, b[0]);
      mlb[i] = lb;
      mom[i] = NSW6_CK(R, 14 + i, mth.exp(fmaR(logX, lb, la)));
    }
    RMOMs_Vt = NSW6_CK(R, 21, mom[5] / mom[2]);
  }
  const R MOMs_0 = mom[0], MOMs_1 = mom[1], MOMs_2 = Xs2;
  const R MOMs_0bs = mom[2], MOMs_1bs = mom[3], MOMs_2bs = mom[4], MOMs_2ds = mom[5];
  const R MOMs_5ds_h = mom[6];

  // graupel slope parameter
  const bool graupel = ge_c(qg, R(1.0E-12));
  R g_a = Z, g_b = Z, g_s1 = Z;
  R RLMDg = Z, RLMDg_dg = Z, RLMDg_2 = Z, RLMDg_3 = Z, RLMDg_3dg = Z, RLMDg_5dg = Z, g32 = Z;
  if (graupel) {
    g_a = densR * qg;
    g_b = g_a * C.K_rlmdg;
    g_s1 = NSW6_CK(R, 22, sqrtR(g_b));
    RLMDg = NSW6_CK(R, 23, sqrtR(g_s1));
    RLMDg_dg = NSW6_CK(R, 24, sqrtR(RLMDg));
    RLMDg_2 = RLMDg * RLMDg;
    RLMDg_3 = RLMDg_2 * RLMDg;
    RLMDg_3dg = RLMDg_3 * RLMDg_dg;
    g32 = RLMDg_3 * RLMDg_2;
    RLMDg_5dg = g32 * RLMDg_dg;
  }

  // terminal velocity
  const R vtr_a = C.K_vtr * rho_fact;
  const R Vtr = vtr_a * RLMDr_dr;
  const R vts_a = C.K_vts * rho_fact;
  const R Vts = vts_a * RMOMs_Vt;
  const R vtg_a = C.K_vtg * rho_fact;
  const R Vtg = vtg_a * RLMDg_dg;

  // nucleation
  const R nm01 = R(-0.1) * temc;
  const R nmax = maxz(nm01);
  const R nex = R(1.33) * (C.ln1000 + nmax);
  const R nexp = NSW6_CK(R, 25, mth.exp(nex));
  const R qi0a = C.ice_nuc * nexp;
  const R Qi0 = qi0a * Rdens;
  const R pg1 = Qi0 - qi, pg2 = qv - qsati;
  const R pgmin = dmin(pg1, pg2);
  const R pgmax = maxz(pgmin);
  R Pigen = pgmax * rdtR;

  // accretion
  R Esi_mod = C.Esi, betai = C.beta_saut, eg = Z;
  bool esi_exp = false, bet_exp = false;   // Esi_mod / betai took the exponential branch of min
  const bool cold_branch = !(warm && is_nonneg(C.Esi) && is_nonneg(C.beta_saut));
  if (cold_branch) {
    eg = NSW6_CK(R, 26, mth.exp(C.gamma_sacr * temc));
    const R es = C.Esi * eg;
    esi_exp = es < C.Esi;
    Esi_mod = esi_exp ? es : C.Esi;
    const R bs = C.beta_saut * eg;   // gamma_saut == gamma_sacr
    bet_exp = bs < C.beta_saut;
    betai = bet_exp ? bs : C.beta_saut;
  }
  const R qcqr = qc * qr;
  R Pracw = Z, prw_pow = Z;
  const bool prw_on = ge_c(qcqr, R(1.0E-12));
  if (prw_on) {
    prw_pow = NSW6_CK(R, 27, mth.pow(qcqr, R(1.15)));
    Pracw = R(67.0) * prw_pow;
  }
  const R fr = rho_fact;
  const R sacw_a = qc * C.K_sacw, sacw_b = sacw_a * MOMs_2ds;
  R Psacw = sacw_b * fr;
  const R gacw_a = qc * C.K_gacw, gacw_b = gacw_a * RLMDg_3dg;
  R Pgacw = gacw_b * fr;
  const R raci_a = qi * C.K_raci, raci_b = raci_a * RLMDr_3dr;
  R Praci = raci_b * fr;
  const R saci_a = qi * C.K_saci, saci_b = saci_a * Esi_mod, saci_c = saci_b * MOMs_2ds;
  R Psaci = saci_c * fr;
  const R iacr_a = qi * C.K_iacr, iacr_b = iacr_a * RLMDr_6dr;
  R Piacr = iacr_b * fr;
  const R dvrs_d = Vtr - Vts;
  const R dvrs = fabsR(dvrs_d);
  const R sacr_k = C.K_sacr * Rdens, sacr_kd = sacr_k * dvrs;
  const R sacr_t1 = C.GAM_1br * RLMDr_1br, sacr_t1m = sacr_t1 * MOMs_2;
  const R sacr_t2 = C.K_2gam2br * RLMDr_2br, sacr_t2m = sacr_t2 * MOMs_1;
  const R sacr_t3 = C.GAM_3br * RLMDr_3br, sacr_t3m = sacr_t3 * MOMs_0;
  const R sacr_s = sacr_t1m + sacr_t2m + sacr_t3m;
  R Psacr = sacr_kd * sacr_s;
  const R dvgr_d = Vtg - Vtr;
  const R dvgr = fabsR(dvgr_d);
  const R gacr_k = C.K_gacr * Rdens, gacr_kd = gacr_k * dvgr;
  const R gacr_t1 = C.K_g13 * RLMDr_1br, gacr_t1m = gacr_t1 * RLMDg_3;
  const R gacr_t2 = C.K_g22 * RLMDr_2br, gacr_t2m = gacr_t2 * RLMDg_2;
  const R gacr_t3 = C.GAM_3br * RLMDr_3br, gacr_t3m = gacr_t3 * RLMDg;
  const R gacr_s = gacr_t1m + gacr_t2m + gacr_t3m;
  R Pgacr = gacr_kd * gacr_s;
  const R racs_k = C.K_racs * Rdens, racs_kd = racs_k * dvrs;
  const R racs_t1 = R(2.0) * MOMs_0bs, racs_t1m = racs_t1 * RLMDr_3;
  const R racs_t2 = R(2.0) * MOMs_1bs, racs_t2m = racs_t2 * RLMDr_2;
  const R racs_t3m = MOMs_2bs * RLMDr;
  const R racs_s = racs_t1m + racs_t2m + racs_t3m;
  R Pracs = racs_kd * racs_s;

  // autoconversion
  const R rhoqc_a = densR * qc;
  const R rhoqc = rhoqc_a * R(1000.0);
  R Praut = Z, aut_pow = Z;
  const bool aut_on = gt_z(qc);
  if (aut_on) {
    aut_pow = NSW6_CK(R, 28, mth.pow(qc, R(2.47)));
    Praut = C.K_aut * aut_pow;
  }
  const R saut_a = qi - C.qicrt_saut;
  const R saut_b = betai * saut_a;
  R Psaut = maxz(saut_b);

  // evaporation, sublimation, melting and freezing
  const R Ka = (R(2.428E-2) + R(7.47E-5) * temc);
  const R kd0 = (R(2.222E-5) + R(1.37E-7) * temc);
  const R kd1 = kd0 * R(PSTD);
  const R kd2 = NSW6_CK(R, 29, kd1 / pre);
  const R KdD = kd2 * densR;
  const R nu0 = (R(1.718E-5) + R(5.28E-8) * temc);
  const R rNu = NSW6_CK(R, 30, densR / nu0);
  const R kat = Ka * tempR;
  const R rKaT = NSW6_CK(R, 31, ONE / kat);
  const R xi = KdD * qsati;
  const R gv1 = R(LHS0) * rKaT;
  const R gv2 = C.LovR_ice * rtem;
  const R gv3 = gv2 - ONE;
  const R gv4 = gv1 * gv3;
  const R gv5 = gv4 * xi;
  const R gv6 = gv5 + ONE;
  const R Giv = NSW6_CK(R, 32, xi / gv6);
  const R gil_a = Ka * temc;
  const R Gil = gil_a * C.rLHF0;
  R Prevp = Z;
  R xl = Z, gl1 = Z, gl2 = Z, gl3 = Z, gl4 = Z, gl5 = Z, gl6 = Z, Glv = Z;
  R vr1 = Z, vr2 = Z, vr3 = Z, vr4 = Z, vr5 = Z, vr6 = Z, ventr = Z;
  R ev1 = Z, ev2 = Z, ev3 = Z, ev4 = Z;
  bool sl_min = false;
  if (rain) {
    xl = KdD * qsatl;
    gl1 = R(LHV0) * rKaT;
    gl2 = C.LovR_liq * rtem;
    gl3 = gl2 - ONE;
    gl4 = gl1 * gl3;
    gl5 = gl4 * xl;
    gl6 = gl5 + ONE;
    Glv = NSW6_CK(R, 33, xl / gl6);
    vr1 = C.K_ventr1 * RLMDr_2;
    vr2 = C.Cr * fr;
    vr3 = vr2 * rNu;
    vr4 = vr3 * RLMDr_5dr;
    vr5 = NSW6_CK(R, 34, sqrtR(vr4));
    vr6 = C.K_ventr2 * vr5;
    ventr = vr1 + vr6;
    ev1 = C.K_revp * Rdens;
    sl_min = !gt_c(Sliq, ONE);   // dmin(Sliq, 1) = Sliq when !(1 < Sliq)
    ev2 = ONE - (sl_min ? Sliq : ONE);
    ev3 = ev1 * ev2;
    ev4 = ev3 * Glv;
    Prevp = ev4 * ventr;
  }
  const R rhoqi_a = densR * qi;
  const bool rqi_on = !lt_c(rhoqi_a, R(EPS));   // dmax(dens qi, EPS) = dens qi
  const R rhoqi = rqi_on ? rhoqi_a : R(EPS);
  R XNi = C.XNi_eps, Di = C.Di_eps;
  R xn_pow = Z, xn_a = Z, XMi = Z, di_s = Z, di_a = Z;
  bool xn_lo = false, xn_hi = false, di_cap = false;
  const bool ice_on = gt_c(rhoqi, R(EPS));
  if (ice_on) {
    xn_pow = NSW6_CK(R, 35, mth.pow(rhoqi, R(0.75)));
    xn_a = R(5.38E+7) * xn_pow;
    xn_lo = lt_c(xn_a, R(1.0E+3));             // dmax(xn_a, 1e3) gives 1e3
    const R xm = xn_lo ? R(1.0E+3) : xn_a;
    xn_hi = gt_c(xm, R(1.0E+6));               // dmin(xm, 1e6) gives 1e6
    XNi = xn_hi ? R(1.0E+6) : xm;
    XMi = NSW6_CK(R, 36, rhoqi / XNi);
    di_s = NSW6_CK(R, 37, sqrtR(XMi));
    di_a = C.Di_a * di_s;
    di_cap = gt_c(di_a, C.Di_max);
    Di = di_cap ? C.Di_max : di_a;
  }
  const R t1a = R(4.0) * Di, t1b = t1a * XNi, t1c = t1b * Rdens, sm1 = Sice - ONE, t1d = t1c * sm1;
  const R tmp1 = t1d * Giv;
  R Pidep = sel(sps, tmp1);
  R Pisub = sel(!sps, -tmp1);
  const bool below40 = lt_z(temc + R(40.0));
  R Pihom = below40 ? dqc_dt : Z;
  const R efa = -C.A_frz * temc;
  const R efe = NSW6_CK(R, 38, mth.exp(efa));
  const R efrz = efe - ONE;
  const bool htr_on = (!below40 && !warm);
  const R qc2 = qc * qc;
  const R ht1 = densR * qc2, ht2 = ht1 * C.K_ihtr;
  R Pihtr = htr_on ? ht2 * efrz : Z;
  R Pimlt = warm ? dqi_dt : Z;
  const R vs1 = R(0.65) * MOMs_1;
  const R vs2 = fr * rNu;
  const R vs3 = NSW6_CK(R, 39, sqrtR(vs2));
  const R vs4 = C.K_vents2 * vs3;
  const R vs5 = vs4 * MOMs_5ds_h;
  const R vents = vs1 + vs5;
  const R s1a = C.K_2pi * Rdens, s1b = s1a * sm1, s1c = s1b * Giv;
  const R tmp2 = s1c * vents;
  R Psdep = sel(sps, tmp2);
  R Pssub = sel(!sps, -tmp2);
  const R sm_a = s1a * Gil, sm_b = sm_a * vents;
  const R sm_c = C.K_clf * temc, sm_d = Psacw + Psacr, sm_e = sm_c * sm_d;
  const R sm_f = sm_b + sm_e;
  R Psmlt = maxz(sm_f);
  const R vg1 = C.K_ventg1 * RLMDg_2;
  const R vg2 = C.Cg * fr, vg3 = vg2 * rNu, vg4 = vg3 * RLMDg_5dg;
  const R vg5 = NSW6_CK(R, 40, sqrtR(vg4));
  const R vg6 = C.K_ventg2 * vg5;
  const R ventg = vg1 + vg6;
  const R g1a = C.K_gdep * Rdens, g1b = g1a * sm1, g1c = g1b * Giv;
  const R tmp3 = g1c * ventg;
  R Pgdep = sel(sps, tmp3);
  R Pgsub = sel(!sps, -tmp3);
  const R gm_a = g1a * Gil, gm_b = gm_a * ventg;
  const R gm_d = Pgacw + Pgacr, gm_e = sm_c * gm_d;
  const R gm_f = gm_b + gm_e;
  R Pgmlt = maxz(gm_f);
  const R gf_a = C.K_gfrz * Rdens, gf_b = gf_a * efrz;
  R Pgfrz = gf_b * RLMDr_7;

  // limiters (:1249-1296); each records which operand of min it took
  const bool cold = !warm;
  const R Pigen0 = Pigen, Pidep0 = Pidep, Psdep0 = Psdep, Pgdep0 = Pgdep;
  Pigen = sel(cold, min_nn(Pigen, dqv_dt));
  Pidep = sel(cold, min_nn(Pidep, dqv_dt));
  Psdep = sel(cold, min_nn(Psdep, dqv_dt));
  Pgdep = sel(cold, min_nn(Pgdep, dqv_dt));
  const R Pracw_a = Pracw + sel(warm, Psacw);
  const R Pracw_b = Pracw_a + sel(warm, Pgacw);
  const R Praut0 = Praut, Pracw0 = Pracw_b, Pihom0 = Pihom, Pihtr0 = Pihtr, Psacw0 = Psacw, Pgacw0 = Pgacw;
  Praut = min_nn(Praut, dqc_dt);
  Pracw = min_nn(Pracw_b, dqc_dt);
  Pihom = sel(cold, min_nn(Pihom, dqc_dt));
  Pihtr = sel(cold, min_nn(Pihtr, dqc_dt));
  Psacw = sel(cold, min_nn(Psacw, dqc_dt));
  Pgacw = sel(cold, min_nn(Pgacw, dqc_dt));
  const R Prevp0 = Prevp, Piacr0 = Piacr, Psacr0 = Psacr, Pgacr0 = Pgacr, Pgfrz0 = Pgfrz;
  Prevp = min_nn(Prevp, dqr_dt);
  Piacr = sel(cold, min_nn(Piacr, dqr_dt));
  Psacr = sel(cold, min_nn(Psacr, dqr_dt));
  Pgacr = sel(cold, min_nn(Pgacr, dqr_dt));
  Pgfrz = sel(cold, min_nn(Pgfrz, dqr_dt));
  const R Pisub0 = Pisub, Pimlt0 = Pimlt, Psaut0 = Psaut, Praci0 = Praci, Psaci0 = Psaci;
  Pisub = sel(cold, min_nn(Pisub, dqi_dt));
  Pimlt = sel(warm, min_nn(Pimlt, dqi_dt));
  Psaut = sel(cold, min_nn(Psaut, dqi_dt));
  Praci = sel(cold, min_nn(Praci, dqi_dt));
  Psaci = sel(cold, min_nn(Psaci, dqi_dt));
  const R Pssub0 = Pssub, Psmlt0 = Psmlt, Pracs0 = Pracs;
  Pssub = sel(cold, min_nn(Pssub, dqs_dt));
  Psmlt = sel(warm, min_nn(Psmlt, dqs_dt));
  Pracs = sel(cold, min_nn(Pracs, dqs_dt));
  const R Pgsub0 = Pgsub, Pgmlt0 = Pgmlt;
  Pgsub = sel(cold, min_nn(Pgsub, dqg_dt));
  Pgmlt = sel(warm, min_nn(Pgmlt, dqg_dt));
  R Piacr_s = sel(!d1, Piacr);
  R Piacr_g = sel(d1, Piacr);
  R Praci_s = sel(!d1, Praci);
  R Praci_g = sel(d1, Praci);
  R Psacr_s = sel(d2b, Psacr);
  R Psacr_g = sel(!d2b, Psacr);
  const R Pracs1 = Pracs;
  Pracs = sel(!d2b, Pracs);

  // loss limiters: fac = 1 when net + EPS >= 0, else min(-dq / net, 1)
  struct Lim {
    R net, fac;
    bool scaled, ratio;   // fac != 1; fac is -dq / net (else 1 from min)
  };
  auto limit = [&](int slot, R net, R dq) {
    Lim L;
    L.net = net;
    if (is_nonneg(net + R(EPS))) {
      L.fac = ONE;
      L.ratio = false;
    } else {
      const R r = NSW6_CK(R, slot, -dq / net);
      L.ratio = !gt_c(r, ONE);
      L.fac = L.ratio ? r : ONE;
    }
    L.scaled = L.fac != ONE;
    return L;
  };
  // [QC]
  const R QC_in[7] = {Pimlt, Praut, Pracw, Pihom, Pihtr, Psacw, Pgacw};
  const Lim Lc = limit(41, +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw, dqc_dt);
  if (Lc.scaled) {
    Pimlt *= Lc.fac; Praut *= Lc.fac; Pracw *= Lc.fac; Pihom *= Lc.fac; Pihtr *= Lc.fac; Psacw *= Lc.fac;
    Pgacw *= Lc.fac;
  }
  // [QI]
  const R QI_in[10] = {Pigen, Pidep, Pihom, Pihtr, Pisub, Pimlt, Psaut, Praci_s, Psaci, Praci_g};
  const Lim Li = limit(42, +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g, dqi_dt);
  if (Li.scaled) {
    Pigen *= Li.fac; Pidep *= Li.fac; Pihom *= Li.fac; Pihtr *= Li.fac; Pisub *= Li.fac; Pimlt *= Li.fac;
    Psaut *= Li.fac; Praci_s *= Li.fac; Psaci *= Li.fac; Praci_g *= Li.fac;
  }
  // [QR]
  const R QR_in[11] = {Praut, Pracw, Psmlt, Pgmlt, Prevp, Piacr_s, Psacr_s, Piacr_g, Psacr_g, Pgacr, Pgfrz};
  const Lim Lr = limit(43, +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz,
                       dqr_dt);
  if (Lr.scaled) {
    Praut *= Lr.fac; Pracw *= Lr.fac; Psmlt *= Lr.fac; Pgmlt *= Lr.fac; Prevp *= Lr.fac; Piacr_s *= Lr.fac;
    Psacr_s *= Lr.fac; Piacr_g *= Lr.fac; Psacr_g *= Lr.fac; Pgacr *= Lr.fac; Pgfrz *= Lr.fac;
  }
  // [QV]
  const R QV_in[8] = {Prevp, Pisub, Pssub, Pgsub, Pigen, Pidep, Psdep, Pgdep};
  const Lim Lv = limit(44, +Prevp + Pisub + Pssub + Pgsub - Pigen - Pidep - Psdep - Pgdep, dqv_dt);
  if (Lv.scaled) {
    Prevp *= Lv.fac; Pisub *= Lv.fac; Pssub *= Lv.fac; Pgsub *= Lv.fac; Pigen *= Lv.fac; Pidep *= Lv.fac;
    Psdep *= Lv.fac; Pgdep *= Lv.fac;
  }
  // [QS]
  const R QS_in[10] = {Psdep, Psacw, Piacr_s, Psacr_s, Psaut, Praci_s, Psaci, Pssub, Psmlt, Pracs};
  const Lim Ls = limit(45, +Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs, dqs_dt);
  if (Ls.scaled) {
    Psdep *= Ls.fac; Psacw *= Ls.fac; Piacr_s *= Ls.fac; Psacr_s *= Ls.fac; Psaut *= Ls.fac; Praci_s *= Ls.fac;
    Psaci *= Ls.fac; Pssub *= Ls.fac; Psmlt *= Ls.fac; Pracs *= Ls.fac;
  }
  // [QG]
  const R QG_in[10] = {Pgdep, Pgacw, Piacr_g, Psacr_g, Pgacr, Pgfrz, Praci_g, Pracs, Pgsub, Pgmlt};
  const Lim Lg = limit(46, +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt, dqg_dt);
  if (Lg.scaled) {
    Pgdep *= Lg.fac; Pgacw *= Lg.fac; Piacr_g *= Lg.fac; Psacr_g *= Lg.fac; Pgacr *= Lg.fac; Pgfrz *= Lg.fac;
    Praci_g *= Lg.fac; Pracs *= Lg.fac; Pgsub *= Lg.fac; Pgmlt *= Lg.fac;
  }

  // tendencies
  const R qc_t0 = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw;
  const R qr_t0 = +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz;
  const R qi_t0 = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g;
  const R qs_t0 = +Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs;
  const R qg_t0 = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt;
  // qx_t = max(qx_t0, -dqx_dt): true when the tendency itself is kept
  const bool kc_ = !lt_nd(qc_t0, dqc_dt), kr_ = !lt_nd(qr_t0, dqr_dt), ki_ = !lt_nd(qi_t0, dqi_dt);
  const bool ks_ = !lt_nd(qs_t0, dqs_dt), kg_ = !lt_nd(qg_t0, dqg_dt);
  const R qc_t = kc_ ? qc_t0 : -dqc_dt, qr_t = kr_ ? qr_t0 : -dqr_dt, qi_t = ki_ ? qi_t0 : -dqi_dt;
  const R qs_t = ks_ ? qs_t0 : -dqs_dt, qg_t = kg_ ? qg_t0 : -dqg_dt;
  const R qv_t = -(qc_t + qr_t + qi_t + qs_t + qg_t);
  const R qt[6] = {qv_t, qc_t, qr_t, qi_t, qs_t, qg_t};
  // budget increments drq = (rhog qt) dt (FP64); in the mixed step a species
  // whose loss reached its whole content leaves exactly nothing (drq = -rq)
  // and the vapour takes the balance (nsw6_cell)
  D drq[6];
  bool exh[6] = {false, false, false, false, false, false};
  if constexpr (kMixed) {
    // formed in FP32 as in nsw6_cell: qt (rhog dt)
    const R rgdt = R(rhog * dt);
    const R lim[6] = {dqv_dt, dqc_dt, dqr_dt, dqi_dt, dqs_dt, dqg_dt};
    D sum = 0.0;
#pragma unroll
    for (int n = 1; n <= 5; ++n) {
      exh[n] = qt[n] <= -lim[n] && lim[n] > Z;
      drq[n] = exh[n] ? -rq[n] : D(qt[n] * rgdt);
      sum += drq[n];
    }
    drq[0] = -sum;
  } else {
#pragma unroll
    for (int n = 0; n < 6; ++n) drq[n] = rhog * D(qt[n]) * dt;
  }
  D rq2[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) rq2[n] = rq[n] + drq[n];
  // effective radius and cloud top
  const R xf1 = rhoqc * C.K_xf;
  const R xf2 = C.coef_xf * xf1;
  const R xf3 = xf2 + R(EPS);
  const R rf_qc = NSW6_CK(R, 47, mth.pow(xf3, R(0.33333333)));
  const R rf2 = rf_qc * rf_qc;
  const R r2_qc = C.K_r2c * rf2;
  const R r2_qr = C.K_r2r * RLMDr_3;
  const R r3c_a = C.coef_xf * densR, r3_qc = r3c_a * qc;
  const R r3_qr = r3c_a * qr;
  const R r2 = r2_qc + r2_qr;
  const bool big = ge_c(r2, R(1.0E-10));
  const R r3 = r3_qc + r3_qr;
  const bool top = !big && ge_c(qc + qr, R(1.0E-5));
  const bool cld = ge_c(r2_qc, R(1.0E-10));
  // updates (FP64)
  const D rhoge1 = rhoge0 - LHV0 * drq[0];
  const D rhoge2 = rhoge1 + LHF0 * drq[3];
  const D rhoge3 = rhoge2 + LHF0 * drq[4];
  const D rhoge = rhoge3 + LHF0 * drq[5];
  D q2[6];
  q2[0] = qn[0];
  D cva = CVDRY, rcva = 0.0, tem_o;
  if constexpr (kMixed) {
    // as nsw6_cell: q from the reciprocal, T = rhoge / (rhog CVdry)
#pragma unroll
    for (int n = 1; n <= 5; ++n) q2[n] = rq2[n] * rrhog;
    tem_o = NSW6_CK(D, 48, rhoge * rrhog * (1.0 / CVDRY));
  } else {
#pragma unroll
    for (int n = 1; n <= 5; ++n) q2[n] = div_rn(rq2[n], rhog, rrhog);
    D qd2 = 1.0;
#pragma unroll
    for (int n = 1; n <= 5; ++n) qd2 = qd2 - q2[n];
    cva = qd2 * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cva = cva + q2[n] * CVDRY;
    rcva = rhog * cva;
    tem_o = NSW6_CK(D, 48, rhoge / rcva);
  }
  if constexpr (MODE == CA_SAVE) {
    // the outputs of nsw6_cell (the same operations on the same values)
    out->Vtr = D(Vtr);
    out->Vts = D(Vts);
    out->Vtg = D(Vtg);
    out->Vti = 0.0;
    out->rceff = big ? D(r3 / r2) : 0.0;
    out->rctop = top ? out->rceff : UNDEF;
    out->tctop = top ? temp : UNDEF;
    out->rceff_cld = cld ? D(r3_qc / r2_qc) : 0.0;
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      out->q[n] = q2[n];
      out->rhogq[n] = rq2[n];
    }
    out->tem = tem_o;
    out->rhog = rhog;
    out->rhoge = rhoge;
    return;
  }

  // ==================================================================== reverse
  // ---- the FP64 updates
  D b_rhog = ob.rhog, b_rhoge = ob.rhoge;
  D b_rq2[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) b_rq2[n] = ob.rhogq[n];
  D b_q2[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) b_q2[n] = ob.q[n];
  // tem_o = rhoge / rcva (mixed: (rhoge / rhog) / CVdry)
  {
    const D g = ob.tem;
    if constexpr (kMixed) {
      b_rhoge = fma(g, rrhog * (1.0 / CVDRY), b_rhoge);
      b_rhog = fma(-g * tem_o, rrhog, b_rhog);
    } else {
      const D rr = 1.0 / rcva;
      b_rhoge = fma(g, rr, b_rhoge);
      const D b_rcva = -g * tem_o * rr;
      b_rhog = fma(b_rcva, cva, b_rhog);
      const D b_cva = b_rcva * rhog;
      // cva = qd2 CV + sum q2 CV
      const D b_qd2 = b_cva * CVDRY;
#pragma unroll
      for (int n = 1; n <= 5; ++n) b_q2[n] += b_cva * CVDRY - b_qd2;
    }
  }
  // q2[n] = rq2[n] / rhog
#pragma unroll
  for (int n = 1; n <= 5; ++n) {
    b_rq2[n] = fma(b_q2[n], rrhog, b_rq2[n]);
    b_rhog = fma(-(b_q2[n] * q2[n]), rrhog, b_rhog);
  }
  // rhoge = rhoge0 - LHV0 drq0 + LHF0 (drq3 + drq4 + drq5); rq2 = rq + drq
  const D b_rhoge0 = b_rhoge;
  D b_drq[6] = {-(b_rhoge * LHV0), 0.0, 0.0, b_rhoge * LHF0, b_rhoge * LHF0, b_rhoge * LHF0};
  D b_rq[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    b_rq[n] = b_rq2[n];
    b_drq[n] += b_rq2[n];
  }
  if constexpr (kMixed) {
    // drq0 = -sum drq[1..5]; drq[n] = -rq[n] for an exhausted species
#pragma unroll
    for (int n = 1; n <= 5; ++n) b_drq[n] -= b_drq[0];
    b_drq[0] = 0.0;
#pragma unroll
    for (int n = 1; n <= 5; ++n)
      if (exh[n]) {
        b_rq[n] -= b_drq[n];
        b_drq[n] = 0.0;
      }
  }
  // drq = (rhog qt) dt
  D b_qtD[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    const D b_rqt = b_drq[n] * dt;
    b_rhog = fma(b_rqt, D(qt[n]), b_rhog);
    b_qtD[n] = b_rqt * rhog;
  }
  // ---- rate precision from here to the psat block.  The sweep is linear in
  // the adjoints that enter it (the tendencies', the fall speeds', the
  // effective radii's); in FP32 they are first scaled by a power of two that
  // brings the largest to [1, 2), and what leaves it is scaled back (exact),
  // so that large output adjoints cannot overflow FP32.
  D sc = 1.0, isc = 1.0;
  if constexpr (kMixed) {
    // the largest biased exponent among them, on the integer pipe
    auto ebits = [](double v) { return (unsigned long long)__double_as_longlong(v) & 0x7ff0000000000000ull; };
    unsigned long long me = ebits(ob.Vtr);
    me = max(me, ebits(ob.Vts));
    me = max(me, ebits(ob.Vtg));
    me = max(me, ebits(ob.rceff));
    me = max(me, ebits(ob.rceff_cld));
#pragma unroll
    for (int n = 0; n < 6; ++n) me = max(me, ebits(b_qtD[n]));
    const int ex = (int)(me >> 52);   // biased exponent of the largest
    if (ex >= 1 && ex <= 2045) {
      sc = __longlong_as_double((long long)(2046 - ex) << 52);   // 2^(1023 - ex)
      isc = __longlong_as_double((long long)ex << 52);           // 2^(ex - 1023)
    }
  }
  R b_qt[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) b_qt[n] = R(b_qtD[n] * sc);
  // effective radius and cloud top: adjoints of the dens, qc, qr, RLMDr_3, temp they read
  R b_dens = Z, b_qc = Z, b_qr = Z, b_RLMDr_3 = Z, b_temp = Z, b_rhoqc = Z;
  D b_tempD = 0.0;   // temp itself (the cloud-top temperature is an FP64 output)
  {
    R b_r2_qc = Z, b_r2_qr = Z, b_r3_qc = Z, b_r3_qr = Z;
    // rceff = big ? r3 / r2 : 0
    if (big) {
      const R rr2 = ONE / r2;
      const R b_r3 = R(ob.rceff * sc) * rr2;
      const R b_r2 = -R(ob.rceff * sc) * (r3 * rr2) * rr2;
      b_r3_qc += b_r3;
      b_r3_qr += b_r3;
      b_r2_qc += b_r2;
      b_r2_qr += b_r2;
    }
    // rctop = top ? rceff (= 0, !big) : UNDEF; tctop = top ? temp : UNDEF
    if (top) b_tempD += ob.tctop;
    // rceff_cld = cld ? r3_qc / r2_qc : 0
    if (cld) {
      const R rr2 = ONE / r2_qc;
      b_r3_qc = fmaR(R(ob.rceff_cld * sc), rr2, b_r3_qc);
      b_r2_qc = fmaR(-(R(ob.rceff_cld * sc) * (r3_qc * rr2)), rr2, b_r2_qc);
    }
    // r3_qc = (coef_xf dens) qc, r3_qr = (coef_xf dens) qr
    b_qc = fmaR(b_r3_qc, r3c_a, b_qc);
    b_qr = fmaR(b_r3_qr, r3c_a, b_qr);
    b_dens = fmaR((b_r3_qc * qc + b_r3_qr * qr), C.coef_xf, b_dens);
    // r2_qr = K_r2r RLMDr_3
    b_RLMDr_3 = fmaR(b_r2_qr, C.K_r2r, b_RLMDr_3);
    // r2_qc = K_r2c rf^2, rf = pow(xf3, 1/3)
    const R b_rf = b_r2_qc * C.K_r2c * R(2.0) * rf_qc;
    const R b_xf3 = gt_z(xf3) ? b_rf * R(0.33333333) * rf_qc / xf3 : Z;
    b_rhoqc = fmaR(b_xf3 * C.coef_xf, C.K_xf, b_rhoqc);
  }
  // Vt outputs
  R b_Vtr = R(ob.Vtr * sc), b_Vts = R(ob.Vts * sc), b_Vtg = R(ob.Vtg * sc);

  // qv_t = -(qc_t + qr_t + qi_t + qs_t + qg_t)
  R b_qc_t = b_qt[1] - b_qt[0], b_qr_t = b_qt[2] - b_qt[0], b_qi_t = b_qt[3] - b_qt[0];
  R b_qs_t = b_qt[4] - b_qt[0], b_qg_t = b_qt[5] - b_qt[0];
  // qx_t = max(qx_t0, -dqx_dt)
  R b_dqv = Z, b_dqc = Z, b_dqr = Z, b_dqi = Z, b_dqs = Z, b_dqg = Z;
  const R b_qc_t0 = kc_ ? b_qc_t : Z;
  if (!kc_) b_dqc -= b_qc_t;
  const R b_qr_t0 = kr_ ? b_qr_t : Z;
  if (!kr_) b_dqr -= b_qr_t;
  const R b_qi_t0 = ki_ ? b_qi_t : Z;
  if (!ki_) b_dqi -= b_qi_t;
  const R b_qs_t0 = ks_ ? b_qs_t : Z;
  if (!ks_) b_dqs -= b_qs_t;
  const R b_qg_t0 = kg_ ? b_qg_t : Z;
  if (!kg_) b_dqg -= b_qg_t;
  // tendency sums: adjoints of the (limited) rates
  R bPimlt = b_qc_t0 - b_qi_t0, bPraut = -b_qc_t0 + b_qr_t0, bPracw = -b_qc_t0 + b_qr_t0;
  R bPihom = -b_qc_t0 + b_qi_t0, bPihtr = -b_qc_t0 + b_qi_t0, bPsacw = -b_qc_t0 + b_qs_t0;
  R bPgacw = -b_qc_t0 + b_qg_t0;
  R bPsmlt = b_qr_t0 - b_qs_t0, bPgmlt = b_qr_t0 - b_qg_t0, bPrevp = -b_qr_t0;
  R bPiacr_s = -b_qr_t0 + b_qs_t0, bPsacr_s = -b_qr_t0 + b_qs_t0, bPiacr_g = -b_qr_t0 + b_qg_t0;
  R bPsacr_g = -b_qr_t0 + b_qg_t0, bPgacr = -b_qr_t0 + b_qg_t0, bPgfrz = -b_qr_t0 + b_qg_t0;
  R bPigen = b_qi_t0, bPidep = b_qi_t0, bPisub = -b_qi_t0, bPsaut = -b_qi_t0 + b_qs_t0;
  R bPraci_s = -b_qi_t0 + b_qs_t0, bPsaci = -b_qi_t0 + b_qs_t0, bPraci_g = -b_qi_t0 + b_qg_t0;
  R bPsdep = b_qs_t0, bPssub = -b_qs_t0, bPracs = -b_qs_t0 + b_qg_t0;
  R bPgdep = b_qg_t0, bPgsub = -b_qg_t0;

  // loss limiters in reverse: x_out = x_in * fac, fac = min(-dq / net, 1), net = sum(+-x_in)
  auto unlimit = [&](const Lim& L, R* const* bx, const R* xin, const R* sgn, int n, R dq, R& b_dq) {
    if (!L.scaled) return;
    R b_fac = Z;
    for (int j = 0; j < n; ++j) {
      b_fac = fmaR(*bx[j], xin[j], b_fac);
      *bx[j] *= L.fac;
    }
    if (L.ratio) {   // fac = -dq / net
      const R rnet = ONE / L.net;
      b_dq = fmaR(-b_fac, rnet, b_dq);
      const R b_net = b_fac * dq * (rnet * rnet);
      for (int j = 0; j < n; ++j) *bx[j] += sgn[j] * b_net;
    }
  };
  {  // [QG]
    R* bx[10] = {&bPgdep, &bPgacw, &bPiacr_g, &bPsacr_g, &bPgacr, &bPgfrz, &bPraci_g, &bPracs, &bPgsub, &bPgmlt};
    const R sg[10] = {1, 1, 1, 1, 1, 1, 1, 1, -1, -1};
    unlimit(Lg, bx, QG_in, sg, 10, dqg_dt, b_dqg);
  }
  {  // [QS]
    R* bx[10] = {&bPsdep, &bPsacw, &bPiacr_s, &bPsacr_s, &bPsaut, &bPraci_s, &bPsaci, &bPssub, &bPsmlt, &bPracs};
    const R sg[10] = {1, 1, 1, 1, 1, 1, 1, -1, -1, -1};
    unlimit(Ls, bx, QS_in, sg, 10, dqs_dt, b_dqs);
  }
  {  // [QV]
    R* bx[8] = {&bPrevp, &bPisub, &bPssub, &bPgsub, &bPigen, &bPidep, &bPsdep, &bPgdep};
    const R sg[8] = {1, 1, 1, 1, -1, -1, -1, -1};
    unlimit(Lv, bx, QV_in, sg, 8, dqv_dt, b_dqv);
  }
  {  // [QR]
    R* bx[11] = {&bPraut, &bPracw, &bPsmlt, &bPgmlt, &bPrevp, &bPiacr_s, &bPsacr_s, &bPiacr_g, &bPsacr_g,
                 &bPgacr, &bPgfrz};
    const R sg[11] = {1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1};
    unlimit(Lr, bx, QR_in, sg, 11, dqr_dt, b_dqr);
  }
  {  // [QI]
    R* bx[10] = {&bPigen, &bPidep, &bPihom, &bPihtr, &bPisub, &bPimlt, &bPsaut, &bPraci_s, &bPsaci, &bPraci_g};
    const R sg[10] = {1, 1, 1, 1, -1, -1, -1, -1, -1, -1};
    unlimit(Li, bx, QI_in, sg, 10, dqi_dt, b_dqi);
  }
  {  // [QC]
    R* bx[7] = {&bPimlt, &bPraut, &bPracw, &bPihom, &bPihtr, &bPsacw, &bPgacw};
    const R sg[7] = {1, -1, -1, -1, -1, -1, -1};
    unlimit(Lc, bx, QC_in, sg, 7, dqc_dt, b_dqc);
  }
  // species splits
  if (d2b) bPracs = Z;   // Pracs = sel(!d2b, Pracs1)
  R bPsacr = (d2b ? bPsacr_s : Z) + (!d2b ? bPsacr_g : Z);
  R bPraci = (!d1 ? bPraci_s : Z) + (d1 ? bPraci_g : Z);
  R bPiacr = (!d1 ? bPiacr_s : Z) + (d1 ? bPiacr_g : Z);
  (void)Pracs1;
  // limiters in reverse: x = sel(on, min(x0, dq))
  auto unmin = [&](bool on, R x0, R dq, R& bx, R& b_dq) {
    if (!on) {
      bx = Z;
      return;
    }
    const R g = bx;
    bx = Z;
    if (lt_nn(dq, x0)) b_dq += g;   // bmin(x0, dq, ...) with dq = max(q, 0) / dt, not negative
    else bx += g;
  };
  unmin(warm, Pgmlt0, dqg_dt, bPgmlt, b_dqg);
  unmin(cold, Pgsub0, dqg_dt, bPgsub, b_dqg);
  unmin(cold, Pracs0, dqs_dt, bPracs, b_dqs);
  unmin(warm, Psmlt0, dqs_dt, bPsmlt, b_dqs);
  unmin(cold, Pssub0, dqs_dt, bPssub, b_dqs);
  unmin(cold, Psaci0, dqi_dt, bPsaci, b_dqi);
  unmin(cold, Praci0, dqi_dt, bPraci, b_dqi);
  unmin(cold, Psaut0, dqi_dt, bPsaut, b_dqi);
  unmin(warm, Pimlt0, dqi_dt, bPimlt, b_dqi);
  unmin(cold, Pisub0, dqi_dt, bPisub, b_dqi);
  unmin(cold, Pgfrz0, dqr_dt, bPgfrz, b_dqr);
  unmin(cold, Pgacr0, dqr_dt, bPgacr, b_dqr);
  unmin(cold, Psacr0, dqr_dt, bPsacr, b_dqr);
  unmin(cold, Piacr0, dqr_dt, bPiacr, b_dqr);
  unmin(true, Prevp0, dqr_dt, bPrevp, b_dqr);
  unmin(cold, Pgacw0, dqc_dt, bPgacw, b_dqc);
  unmin(cold, Psacw0, dqc_dt, bPsacw, b_dqc);
  unmin(cold, Pihtr0, dqc_dt, bPihtr, b_dqc);
  unmin(cold, Pihom0, dqc_dt, bPihom, b_dqc);
  unmin(true, Pracw0, dqc_dt, bPracw, b_dqc);
  unmin(true, Praut0, dqc_dt, bPraut, b_dqc);
  // Pracw_b = Pracw + sel(warm, Psacw) + sel(warm, Pgacw) (before their own limits)
  R bPracw0 = bPracw;
  R bPsacw_w = warm ? bPracw : Z, bPgacw_w = warm ? bPracw : Z;
  bPsacw += bPsacw_w;
  bPgacw += bPgacw_w;
  unmin(cold, Pgdep0, dqv_dt, bPgdep, b_dqv);
  unmin(cold, Psdep0, dqv_dt, bPsdep, b_dqv);
  unmin(cold, Pidep0, dqv_dt, bPidep, b_dqv);
  unmin(cold, Pigen0, dqv_dt, bPigen, b_dqv);

  // ---- process rates in reverse
  R b_rho_fact = Z, b_Rdens = Z, b_temc = Z, b_rNu = Z, b_Giv = Z, b_Gil = Z, b_Sice = Z;
  R b_Sliq = Z, b_qv = Z, b_qi = Z, b_qs = Z, b_qg = Z, b_qsati = Z, b_qsatl = Z;
  R b_RLMDr = Z, b_RLMDr_dr = Z, b_RLMDr_2 = Z, b_RLMDr_1br = Z, b_RLMDr_2br = Z;
  R b_RLMDr_3br = Z, b_RLMDr_7 = Z, b_RLMDr_3dr = Z, b_RLMDr_5dr = Z, b_RLMDr_6dr = Z;
  R b_RLMDg = Z, b_RLMDg_dg = Z, b_RLMDg_2 = Z, b_RLMDg_3 = Z, b_RLMDg_3dg = Z, b_RLMDg_5dg = Z;
  R b_mom[7] = {Z, Z, Z, Z, Z, Z, Z};
  R b_MOMs_2 = Z, b_RMOMs_Vt = Z, b_Esi_mod = Z, b_betai = Z, b_efrz = Z, b_pre = Z, b_rtem = Z;
  R b_KdD = Z, b_Ka = Z, b_Di = Z, b_XNi = Z, b_rhoqi = Z;
  // parameter-dependent constants
  R b_K_vtr = Z, b_K_raci = Z, b_K_iacr = Z, b_Cr = Z, b_K_vts = Z, b_K_sacw = Z, b_K_saci = Z;
  R b_K_vents2 = Z, b_K_vtg = Z, b_K_gacw = Z, b_Cg = Z, b_beta = Z, b_qicrt = Z, b_icenuc = Z;
  R b_K_aut = Z;

  // Pgfrz = (K_gfrz Rdens) efrz RLMDr_7
  b_Rdens = fmaR(bPgfrz * RLMDr_7 * efrz, C.K_gfrz, b_Rdens);
  b_efrz = fmaR(bPgfrz * RLMDr_7, gf_a, b_efrz);
  b_RLMDr_7 = fmaR(bPgfrz, gf_b, b_RLMDr_7);
  // Pgmlt = max(gm_b + sm_c gm_d, 0); gm_b = (g1a Gil) ventg; gm_d = Pgacw + Pgacr
  R b_ventg = Z, b_g1a = Z, b_sm_c = Z;
  {
    R b_f = Z, dummy = Z;
    bmaxz(gm_f, bPgmlt, b_f, dummy);
    b_g1a = fmaR(b_f * ventg, Gil, b_g1a);
    b_Gil = fmaR(b_f * ventg, g1a, b_Gil);
    b_ventg = fmaR(b_f, gm_a, b_ventg);
    b_sm_c = fmaR(b_f, gm_d, b_sm_c);
    bPgacw = fmaR(b_f, sm_c, bPgacw);
    bPgacr = fmaR(b_f, sm_c, bPgacr);
  }
  // Pgdep = sel(sps, tmp3), Pgsub = sel(!sps, -tmp3); tmp3 = (g1a sm1 Giv) ventg
  {
    const R b_t = (sps ? bPgdep : Z) - (!sps ? bPgsub : Z);
    b_g1a = fmaR(b_t * ventg * Giv, sm1, b_g1a);
    b_Sice = fmaR(b_t * ventg * Giv, g1a, b_Sice);
    b_Giv = fmaR(b_t * ventg, g1b, b_Giv);
    b_ventg = fmaR(b_t, g1c, b_ventg);
  }
  // g1a = K_gdep Rdens
  b_Rdens = fmaR(b_g1a, C.K_gdep, b_Rdens);
  // ventg = K_ventg1 RLMDg_2 + K_ventg2 sqrt(Cg fr rNu RLMDg_5dg)
  {
    b_RLMDg_2 = fmaR(b_ventg, C.K_ventg1, b_RLMDg_2);
    const R b_vg5 = b_ventg * C.K_ventg2;
    const R b_vg4 = b_vg5 * bsqrt(vg5);
    b_RLMDg_5dg = fmaR(b_vg4, vg3, b_RLMDg_5dg);
    const R b_vg3 = b_vg4 * RLMDg_5dg;
    b_rNu = fmaR(b_vg3, vg2, b_rNu);
    const R b_vg2 = b_vg3 * rNu;
    b_Cg = fmaR(b_vg2, fr, b_Cg);
    b_rho_fact = fmaR(b_vg2, C.Cg, b_rho_fact);
  }
  // Psmlt = max(sm_b + sm_c sm_d, 0); sm_b = (s1a Gil) vents; sm_d = Psacw + Psacr
  R b_vents = Z, b_s1a = Z;
  {
    R b_f = Z, dummy = Z;
    bmaxz(sm_f, bPsmlt, b_f, dummy);
    b_s1a = fmaR(b_f * vents, Gil, b_s1a);
    b_Gil = fmaR(b_f * vents, s1a, b_Gil);
    b_vents = fmaR(b_f, sm_a, b_vents);
    b_sm_c = fmaR(b_f, sm_d, b_sm_c);
    bPsacw = fmaR(b_f, sm_c, bPsacw);
    bPsacr = fmaR(b_f, sm_c, bPsacr);
  }
  // sm_c = K_clf temc
  b_temc = fmaR(b_sm_c, C.K_clf, b_temc);
  // Psdep / Pssub: tmp2 = (s1a sm1 Giv) vents
  {
    const R b_t = (sps ? bPsdep : Z) - (!sps ? bPssub : Z);
    b_s1a = fmaR(b_t * vents * Giv, sm1, b_s1a);
    b_Sice = fmaR(b_t * vents * Giv, s1a, b_Sice);
    b_Giv = fmaR(b_t * vents, s1b, b_Giv);
    b_vents = fmaR(b_t, s1c, b_vents);
  }
  b_Rdens = fmaR(b_s1a, C.K_2pi, b_Rdens);
  // vents = 0.65 MOMs_1 + (K_vents2 sqrt(fr rNu)) MOMs_5ds_h
  {
    b_mom[1] = fmaR(b_vents, R(0.65), b_mom[1]);
    b_mom[6] = fmaR(b_vents, vs4, b_mom[6]);
    const R b_vs4 = b_vents * MOMs_5ds_h;
    b_K_vents2 = fmaR(b_vs4, vs3, b_K_vents2);
    const R b_vs2 = b_vs4 * C.K_vents2 * bsqrt(vs3);
    b_rho_fact = fmaR(b_vs2, rNu, b_rho_fact);
    b_rNu = fmaR(b_vs2, fr, b_rNu);
  }
  // Pimlt = warm ? dqi_dt : 0
  if (warm) b_dqi += bPimlt;
  // Pihtr = htr_on ? (dens qc^2 K_ihtr) efrz : 0
  if (htr_on) {
    b_efrz = fmaR(bPihtr, ht2, b_efrz);
    const R b_ht1 = bPihtr * efrz * C.K_ihtr;
    b_dens = fmaR(b_ht1, qc2, b_dens);
    b_qc = fmaR(b_ht1 * densR * R(2.0), qc, b_qc);
  }
  // efrz = exp(-A_frz temc) - 1
  b_temc = fmaR(b_efrz * efe, (-C.A_frz), b_temc);
  // Pihom = below40 ? dqc_dt : 0
  if (below40) b_dqc += bPihom;
  // Pidep / Pisub: tmp1 = (((4 Di) XNi) Rdens sm1) Giv
  {
    const R b_t = (sps ? bPidep : Z) - (!sps ? bPisub : Z);
    b_Giv = fmaR(b_t, t1d, b_Giv);
    const R b_t1d = b_t * Giv;
    b_Sice = fmaR(b_t1d, t1c, b_Sice);
    const R b_t1c = b_t1d * sm1;
    b_Rdens = fmaR(b_t1c, t1b, b_Rdens);
    const R b_t1b = b_t1c * Rdens;
    b_XNi = fmaR(b_t1b, t1a, b_XNi);
    b_Di = fmaR(b_t1b * XNi, R(4.0), b_Di);
  }
  // XNi, Di from rhoqi
  if (ice_on) {
    if (!di_cap) {
      const R b_dia = b_Di;
      const R b_dis = b_dia * C.Di_a;
      const R b_XMi = b_dis * bsqrt(di_s);
      const R rXNi = ONE / XNi;
      b_rhoqi = fmaR(b_XMi, rXNi, b_rhoqi);
      b_XNi = fmaR(-(b_XMi * XMi), rXNi, b_XNi);
    }
    // XNi = min(max(5.38e7 pow(rhoqi, 0.75), 1e3), 1e6)
    if (!xn_hi && !xn_lo) {
      const R b_pow = b_XNi * R(5.38E+7);
      if (gt_z(rhoqi)) b_rhoqi += b_pow * R(0.75) * xn_pow / rhoqi;
    }
  }
  if (rqi_on) {
    b_dens = fmaR(b_rhoqi, qi, b_dens);
    b_qi = fmaR(b_rhoqi, densR, b_qi);
  }
  // Prevp = (((K_revp Rdens) (1 - min(Sliq, 1))) Glv) ventr
  if (rain) {
    const R b_ventr = bPrevp * ev4;
    const R b_ev4 = bPrevp * ventr;
    const R b_Glv = b_ev4 * ev3;
    const R b_ev3 = b_ev4 * Glv;
    const R b_ev1 = b_ev3 * ev2;
    const R b_ev2 = b_ev3 * ev1;
    if (sl_min) b_Sliq -= b_ev2;
    b_Rdens = fmaR(b_ev1, C.K_revp, b_Rdens);
    // ventr = K_ventr1 RLMDr_2 + K_ventr2 sqrt(Cr fr rNu RLMDr_5dr)
    b_RLMDr_2 = fmaR(b_ventr, C.K_ventr1, b_RLMDr_2);
    const R b_vr4 = b_ventr * C.K_ventr2 * bsqrt(vr5);
    b_RLMDr_5dr = fmaR(b_vr4, vr3, b_RLMDr_5dr);
    const R b_vr3 = b_vr4 * RLMDr_5dr;
    b_rNu = fmaR(b_vr3, vr2, b_rNu);
    const R b_vr2 = b_vr3 * rNu;
    b_Cr = fmaR(b_vr2, fr, b_Cr);
    b_rho_fact = fmaR(b_vr2, C.Cr, b_rho_fact);
    // Glv = xl / (((LHV0 rKaT) (LovR_liq rtem - 1)) xl + 1)
    const R rgl6 = ONE / gl6;
    const R b_xl0 = b_Glv * rgl6;
    const R b_gl6 = -b_Glv * Glv * rgl6;
    const R b_gl4 = b_gl6 * xl;
    const R b_xl = b_xl0 + b_gl6 * gl4;
    const R b_gl1 = b_gl4 * gl3;
    const R b_gl3 = b_gl4 * gl1;
    b_rtem = fmaR(b_gl3, C.LovR_liq, b_rtem);
    const R b_rKaT_l = b_gl1 * R(LHV0);
    // xl = KdD qsatl
    b_KdD = fmaR(b_xl, qsatl, b_KdD);
    b_qsatl = fmaR(b_xl, KdD, b_qsatl);
    // rKaT = 1 / (Ka temp)
    const R b_kat = -b_rKaT_l * rKaT * rKaT;
    b_Ka = fmaR(b_kat, tempR, b_Ka);
    b_temp = fmaR(b_kat, Ka, b_temp);
  }
  // Gil = (Ka temc) rLHF0
  {
    const R b_gila = b_Gil * C.rLHF0;
    b_Ka = fmaR(b_gila, temc, b_Ka);
    b_temc = fmaR(b_gila, Ka, b_temc);
  }
  // Giv = xi / (((LHS0 rKaT) (LovR_ice rtem - 1)) xi + 1)
  {
    const R rgv6 = ONE / gv6;
    const R b_xi0 = b_Giv * rgv6;
    const R b_gv6 = -b_Giv * Giv * rgv6;
    const R b_gv4 = b_gv6 * xi;
    const R b_xi = b_xi0 + b_gv6 * gv4;
    const R b_gv1 = b_gv4 * gv3;
    const R b_gv3 = b_gv4 * gv1;
    b_rtem = fmaR(b_gv3, C.LovR_ice, b_rtem);
    const R b_rKaT = b_gv1 * R(LHS0);
    const R b_kat = -b_rKaT * rKaT * rKaT;
    b_Ka = fmaR(b_kat, tempR, b_Ka);
    b_temp = fmaR(b_kat, Ka, b_temp);
    b_KdD = fmaR(b_xi, qsati, b_KdD);
    b_qsati = fmaR(b_xi, KdD, b_qsati);
  }
  // rNu = dens / nu0, nu0 = 1.718e-5 + 5.28e-8 temc
  {
    const R rnu0 = ONE / nu0;
    b_dens = fmaR(b_rNu, rnu0, b_dens);
    const R b_nu0 = -b_rNu * rNu * rnu0;
    b_temc = fmaR(b_nu0, R(5.28E-8), b_temc);
  }
  // KdD = ((kd0 PSTD) / pre) dens, kd0 = 2.222e-5 + 1.37e-7 temc
  {
    b_dens = fmaR(b_KdD, kd2, b_dens);
    const R b_kd2 = b_KdD * densR;
    const R rpre = ONE / pre;
    const R b_kd1 = b_kd2 * rpre;
    b_pre = fmaR(-(b_kd2 * kd2), rpre, b_pre);
    b_temc = fmaR(b_kd1 * R(PSTD), R(1.37E-7), b_temc);
  }
  // Ka = 2.428e-2 + 7.47e-5 temc
  b_temc = fmaR(b_Ka, R(7.47E-5), b_temc);
  // Psaut = max(betai (qi - qicrt), 0), off where its argument is exactly 0
  // (rate_on: a cell without ice at the threshold qicrt = 0)
  {
    const R b_sb = gt_z(saut_b) ? bPsaut : Z;
    b_betai = fmaR(b_sb, saut_a, b_betai);
    const R b_sa = b_sb * betai;
    b_qi += b_sa;
    b_qicrt -= b_sa;
  }
  // Praut = K_aut pow(qc, 2.47)
  if (aut_on) {
    b_K_aut = fmaR(bPraut, aut_pow, b_K_aut);
    if (gt_z(qc)) b_qc += bPraut * C.K_aut * R(2.47) * aut_pow / qc;
  }
  // rhoqc = (dens qc) 1000 (read by the effective radius)
  b_dens = fmaR(b_rhoqc * R(1000.0), qc, b_dens);
  b_qc = fmaR(b_rhoqc * R(1000.0), densR, b_qc);
  // Pracs = (K_racs Rdens) dvrs (2 MOMs_0bs RLMDr_3 + 2 MOMs_1bs RLMDr_2 + MOMs_2bs RLMDr)
  R b_dvrs = Z;
  {
    const R b_s = bPracs * racs_kd;
    const R b_kd = bPracs * racs_s;
    b_dvrs = fmaR(b_kd, racs_k, b_dvrs);
    b_Rdens = fmaR(b_kd * dvrs, C.K_racs, b_Rdens);
    b_mom[2] = fmaR(b_s * RLMDr_3, R(2.0), b_mom[2]);
    b_RLMDr_3 = fmaR(b_s, racs_t1, b_RLMDr_3);
    b_mom[3] = fmaR(b_s * RLMDr_2, R(2.0), b_mom[3]);
    b_RLMDr_2 = fmaR(b_s, racs_t2, b_RLMDr_2);
    b_mom[4] = fmaR(b_s, RLMDr, b_mom[4]);
    b_RLMDr = fmaR(b_s, MOMs_2bs, b_RLMDr);
  }
  // Pgacr = (K_gacr Rdens) |Vtg - Vtr| (K_g13 RLMDr_1br RLMDg_3 + K_g22 RLMDr_2br RLMDg_2 + GAM_3br RLMDr_3br RLMDg)
  {
    const R b_s = bPgacr * gacr_kd;
    const R b_kd = bPgacr * gacr_s;
    const R b_dv = b_kd * gacr_k;
    b_Rdens = fmaR(b_kd * dvgr, C.K_gacr, b_Rdens);
    const R sgn = lt_z(dvgr_d) ? -ONE : ONE;
    b_Vtg = fmaR(b_dv, sgn, b_Vtg);
    b_Vtr = fmaR(-b_dv, sgn, b_Vtr);
    b_RLMDr_1br = fmaR(b_s * RLMDg_3, C.K_g13, b_RLMDr_1br);
    b_RLMDg_3 = fmaR(b_s, gacr_t1, b_RLMDg_3);
    b_RLMDr_2br = fmaR(b_s * RLMDg_2, C.K_g22, b_RLMDr_2br);
    b_RLMDg_2 = fmaR(b_s, gacr_t2, b_RLMDg_2);
    b_RLMDr_3br = fmaR(b_s * RLMDg, C.GAM_3br, b_RLMDr_3br);
    b_RLMDg = fmaR(b_s, gacr_t3, b_RLMDg);
  }
  // Psacr = (K_sacr Rdens) dvrs (GAM_1br RLMDr_1br MOMs_2 + K_2gam2br RLMDr_2br MOMs_1 + GAM_3br RLMDr_3br MOMs_0)
  {
    const R b_s = bPsacr * sacr_kd;
    const R b_kd = bPsacr * sacr_s;
    b_dvrs = fmaR(b_kd, sacr_k, b_dvrs);
    b_Rdens = fmaR(b_kd * dvrs, C.K_sacr, b_Rdens);
    b_RLMDr_1br = fmaR(b_s * MOMs_2, C.GAM_1br, b_RLMDr_1br);
    b_MOMs_2 = fmaR(b_s, sacr_t1, b_MOMs_2);
    b_RLMDr_2br = fmaR(b_s * MOMs_1, C.K_2gam2br, b_RLMDr_2br);
    b_mom[1] = fmaR(b_s, sacr_t2, b_mom[1]);
    b_RLMDr_3br = fmaR(b_s * MOMs_0, C.GAM_3br, b_RLMDr_3br);
    b_mom[0] = fmaR(b_s, sacr_t3, b_mom[0]);
  }
  // dvrs = |Vtr - Vts|
  {
    const R sgn = lt_z(dvrs_d) ? -ONE : ONE;
    b_Vtr = fmaR(b_dvrs, sgn, b_Vtr);
    b_Vts = fmaR(-b_dvrs, sgn, b_Vts);
  }
  // Piacr = ((qi K_iacr) RLMDr_6dr) fr
  b_rho_fact = fmaR(bPiacr, iacr_b, b_rho_fact);
  {
    const R b_b = bPiacr * fr;
    b_RLMDr_6dr = fmaR(b_b, iacr_a, b_RLMDr_6dr);
    const R b_a = b_b * RLMDr_6dr;
    b_qi = fmaR(b_a, C.K_iacr, b_qi);
    b_K_iacr = fmaR(b_a, qi, b_K_iacr);
  }
  // Psaci = (((qi K_saci) Esi_mod) MOMs_2ds) fr
  b_rho_fact = fmaR(bPsaci, saci_c, b_rho_fact);
  {
    const R b_c = bPsaci * fr;
    b_mom[5] = fmaR(b_c, saci_b, b_mom[5]);
    const R b_b = b_c * MOMs_2ds;
    b_Esi_mod = fmaR(b_b, saci_a, b_Esi_mod);
    const R b_a = b_b * Esi_mod;
    b_qi = fmaR(b_a, C.K_saci, b_qi);
    b_K_saci = fmaR(b_a, qi, b_K_saci);
  }
  // Praci = ((qi K_raci) RLMDr_3dr) fr
  b_rho_fact = fmaR(bPraci, raci_b, b_rho_fact);
  {
    const R b_b = bPraci * fr;
    b_RLMDr_3dr = fmaR(b_b, raci_a, b_RLMDr_3dr);
    const R b_a = b_b * RLMDr_3dr;
    b_qi = fmaR(b_a, C.K_raci, b_qi);
    b_K_raci = fmaR(b_a, qi, b_K_raci);
  }
  // Pgacw = ((qc K_gacw) RLMDg_3dg) fr
  b_rho_fact = fmaR(bPgacw, gacw_b, b_rho_fact);
  {
    const R b_b = bPgacw * fr;
    b_RLMDg_3dg = fmaR(b_b, gacw_a, b_RLMDg_3dg);
    const R b_a = b_b * RLMDg_3dg;
    b_qc = fmaR(b_a, C.K_gacw, b_qc);
    b_K_gacw = fmaR(b_a, qc, b_K_gacw);
  }
  // Psacw = ((qc K_sacw) MOMs_2ds) fr
  b_rho_fact = fmaR(bPsacw, sacw_b, b_rho_fact);
  {
    const R b_b = bPsacw * fr;
    b_mom[5] = fmaR(b_b, sacw_a, b_mom[5]);
    const R b_a = b_b * MOMs_2ds;
    b_qc = fmaR(b_a, C.K_sacw, b_qc);
    b_K_sacw = fmaR(b_a, qc, b_K_sacw);
  }
  // Pracw = 67 pow(qc qr, 1.15)
  if (prw_on) {
    const R b_pow = bPracw0 * R(67.0);
    if (gt_z(qcqr)) {
      const R b_qcqr = b_pow * R(1.15) * prw_pow / qcqr;
      b_qc = fmaR(b_qcqr, qr, b_qc);
      b_qr = fmaR(b_qcqr, qc, b_qr);
    }
  }
  // Esi_mod = min(Esi, Esi eg), betai = min(beta, beta eg), eg = exp(gamma_sacr temc)
  if (cold_branch) {
    R b_eg = Z;
    if (esi_exp) b_eg += b_Esi_mod * C.Esi;
    if (bet_exp) {
      b_eg = fmaR(b_betai, C.beta_saut, b_eg);
      b_beta = fmaR(b_betai, eg, b_beta);
    } else {
      b_beta += b_betai;
    }
    b_temc = fmaR(b_eg * eg, C.gamma_sacr, b_temc);
  } else {
    b_beta += b_betai;
  }
  // Pigen = max(min(Qi0 - qi, qv - qsati), 0) rdt
  {
    const R b_max = bPigen * rdtR;
    R b_min = Z, dummy = Z;
    bmaxz(pgmin, b_max, b_min, dummy);
    R b_p1 = Z, b_p2 = Z;
    bmin(pg1, pg2, b_min, b_p1, b_p2);
    b_qi -= b_p1;
    b_qv += b_p2;
    b_qsati -= b_p2;
    // Qi0 = (ice_nuc exp(1.33 (ln1000 + max(-0.1 temc, 0)))) Rdens
    b_Rdens = fmaR(b_p1, qi0a, b_Rdens);
    const R b_qi0a = b_p1 * Rdens;
    b_icenuc = fmaR(b_qi0a, nexp, b_icenuc);
    const R b_nex = b_qi0a * C.ice_nuc * nexp;
    R b_nm01 = Z, dummy2 = Z;
    bmaxz(nm01, b_nex * R(1.33), b_nm01, dummy2);
    b_temc = fmaR(b_nm01, R(-0.1), b_temc);
  }
  // terminal velocities: Vtr = (K_vtr rho_fact) RLMDr_dr etc.
  {
    b_RLMDr_dr = fmaR(b_Vtr, vtr_a, b_RLMDr_dr);
    const R b_a = b_Vtr * RLMDr_dr;
    b_K_vtr = fmaR(b_a, rho_fact, b_K_vtr);
    b_rho_fact = fmaR(b_a, C.K_vtr, b_rho_fact);
    b_RMOMs_Vt = fmaR(b_Vts, vts_a, b_RMOMs_Vt);
    const R b_s = b_Vts * RMOMs_Vt;
    b_K_vts = fmaR(b_s, rho_fact, b_K_vts);
    b_rho_fact = fmaR(b_s, C.K_vts, b_rho_fact);
    b_RLMDg_dg = fmaR(b_Vtg, vtg_a, b_RLMDg_dg);
    const R b_g = b_Vtg * RLMDg_dg;
    b_K_vtg = fmaR(b_g, rho_fact, b_K_vtg);
    b_rho_fact = fmaR(b_g, C.K_vtg, b_rho_fact);
  }
  // graupel slope parameter
  if (graupel) {
    b_RLMDg_3 = fmaR(b_RLMDg_5dg * RLMDg_dg, RLMDg_2, b_RLMDg_3);
    b_RLMDg_2 = fmaR(b_RLMDg_5dg * RLMDg_dg, RLMDg_3, b_RLMDg_2);
    b_RLMDg_dg = fmaR(b_RLMDg_5dg, g32, b_RLMDg_dg);
    b_RLMDg_3 = fmaR(b_RLMDg_3dg, RLMDg_dg, b_RLMDg_3);
    b_RLMDg_dg = fmaR(b_RLMDg_3dg, RLMDg_3, b_RLMDg_dg);
    b_RLMDg_2 = fmaR(b_RLMDg_3, RLMDg, b_RLMDg_2);
    b_RLMDg = fmaR(b_RLMDg_3, RLMDg_2, b_RLMDg);
    b_RLMDg = fmaR(b_RLMDg_2 * R(2.0), RLMDg, b_RLMDg);
    b_RLMDg = fmaR(b_RLMDg_dg, bsqrt(RLMDg_dg), b_RLMDg);
    const R b_s1 = b_RLMDg * bsqrt(RLMDg);
    const R b_b = b_s1 * bsqrt(g_s1);
    const R b_a = b_b * C.K_rlmdg;
    b_dens = fmaR(b_a, qg, b_dens);
    b_qg = fmaR(b_a, densR, b_qg);
  }
  // snow moments: Vts's RMOMs_Vt = mom5 / mom2; mom_i = exp(logX lb_i + la_i(tems)); MOMs_2 = Xs2
  R b_Xs2 = b_MOMs_2;
  if (snow) {
    const R rm2 = ONE / mom[2];
    b_mom[5] = fmaR(b_RMOMs_Vt, rm2, b_mom[5]);
    b_mom[2] = fmaR(-(b_RMOMs_Vt * RMOMs_Vt), rm2, b_mom[2]);
    R b_logX = Z, b_tems = Z;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const R b_arg = b_mom[i] * mom[i];
      b_logX = fmaR(b_arg, mlb[i], b_logX);
      const R* a = C.roh_a + 4 * i;
      const R* b = C.roh_b + 4 * i;
      // d la / d tems and d lb / d tems of the cubics
      const R dla = fmaR(fmaR(R(3.0) * a[3], tems, R(2.0) * a[2]), tems, a[1]);
      const R dlb = fmaR(fmaR(R(3.0) * b[3], tems, R(2.0) * b[2]), tems, b[1]);
      b_tems = fmaR(b_arg, (dla + logX * dlb), b_tems);
    }
    b_Xs2 += b_logX / Xs2;
    if (tems_sel) b_temc += b_tems;
  }
  {
    const R b_xsa = b_Xs2 * C.rAs;
    b_dens = fmaR(b_xsa, qs, b_dens);
    b_qs = fmaR(b_xsa, densR, b_qs);
  }
  // rain slope parameter
  if (rain) {
    b_RLMDr_3br = fmaR(b_RLMDr_6dr, RLMDr_dr, b_RLMDr_3br);
    b_RLMDr_dr = fmaR(b_RLMDr_6dr, RLMDr_3br, b_RLMDr_dr);
    b_RLMDr_2br = fmaR(b_RLMDr_5dr, RLMDr_dr, b_RLMDr_2br);
    b_RLMDr_dr = fmaR(b_RLMDr_5dr, RLMDr_2br, b_RLMDr_dr);
    b_RLMDr_3 = fmaR(b_RLMDr_3dr, RLMDr_dr, b_RLMDr_3);
    b_RLMDr_dr = fmaR(b_RLMDr_3dr, RLMDr_3, b_RLMDr_dr);
    b_RLMDr_3br = fmaR(b_RLMDr_7, RLMDr, b_RLMDr_3br);
    b_RLMDr = fmaR(b_RLMDr_7, RLMDr_3br, b_RLMDr);
    b_RLMDr_3 = fmaR(b_RLMDr_3br * R(2.0), RLMDr_3, b_RLMDr_3);
    b_RLMDr_1br = fmaR(b_RLMDr_2br, RLMDr, b_RLMDr_1br);
    b_RLMDr = fmaR(b_RLMDr_2br, RLMDr_1br, b_RLMDr);
    b_RLMDr_2 = fmaR(b_RLMDr_1br * R(2.0), RLMDr_2, b_RLMDr_2);
    b_RLMDr_2 = fmaR(b_RLMDr_3, RLMDr, b_RLMDr_2);
    b_RLMDr = fmaR(b_RLMDr_3, RLMDr_2, b_RLMDr);
    b_RLMDr = fmaR(b_RLMDr_2 * R(2.0), RLMDr, b_RLMDr);
    b_RLMDr = fmaR(b_RLMDr_dr, bsqrt(RLMDr_dr), b_RLMDr);
    const R b_s1 = b_RLMDr * bsqrt(RLMDr);
    const R b_b = b_s1 * bsqrt(r_s1);
    const R b_a = b_b * C.K_rlmdr;
    b_dens = fmaR(b_a, qr, b_dens);
    b_qr = fmaR(b_a, densR, b_qr);
  }
  // dq/dt = q / dt
  b_qv = fmaR(b_dqv, rdtR, b_qv);
  b_qc = fmaR(b_dqc, rdtR, b_qc);
  b_qr = fmaR(b_dqr, rdtR, b_qr);
  b_qi = fmaR(b_dqi, rdtR, b_qi);
  b_qs = fmaR(b_dqs, rdtR, b_qs);
  b_qg = fmaR(b_dqg, rdtR, b_qg);
  // temc = temp - TEM00; rho_fact = sqrt(DENS00 Rdens); Rdens = 1 / dens
  b_temp += b_temc;
  b_Rdens = fmaR(b_rho_fact * bsqrt(rho_fact), R(DENS00), b_Rdens);
  b_dens = fmaR(-(b_Rdens * Rdens), Rdens, b_dens);
  // Sliq = qv / max(qsatl, EPS), Sice = qv / max(qsati, EPS)
  {
    const R rsld = ONE / sld;
    b_qv = fmaR(b_Sliq, rsld, b_qv);
    const R b_sld = -b_Sliq * Sliq * rsld;
    R dummy = Z;
    bmaxc(qsatl, R(EPS), b_sld, b_qsatl, dummy);
    const R rsid = ONE / sid;
    b_qv = fmaR(b_Sice, rsid, b_qv);
    const R b_sid = -b_Sice * Sice * rsid;
    bmaxc(qsati, R(EPS), b_sid, b_qsati, dummy);
  }
  // q* = max(qn, 0) (compared in the rate precision, as the forward does)
  D b_qn[6] = {0, 0, 0, 0, 0, 0};
  {
    const R bq[6] = {b_qv, b_qc, b_qr, b_qi, b_qs, b_qg};
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      R b = Z, dummy = Z;
      bmaxz(R(qn[n]), bq[n], b, dummy);
      b_qn[n] = D(b) * isc;
    }
  }
  // psat / qsat: qsat = psat (1 / ((dens RVAP) temp)), psat = PSAT0 exp(LovR (RTEM00 - rtem))
  {
    const R b_rdrt = b_qsatl * psatl + b_qsati * psati;
    const R b_psatl = b_qsatl * rdrt, b_psati = b_qsati * rdrt;
    const R b_drt = -b_rdrt * rdrt * rdrt;
    b_dens = fmaR(b_drt * tempR, R(RVAP), b_dens);
    b_temp = fmaR(b_drt, drv, b_temp);
    b_rtem -= b_psatl * R(PSAT0) * el * C.LovR_liq + b_psati * R(PSAT0) * ei * C.LovR_ice;
    // rtem = 1 / max(temp, TEM_MIN)
    const R b_tmx = -b_rtem * rtem * rtem;
    R dummy = Z;
    bmaxc(tempR, R(TEM_MIN), b_tmx, b_temp, dummy);
  }
  // ---- FP64 from here: pre = (dens (qd RDRY + qn0 RVAP)) temp
  D b_densD = D(b_dens) * isc;
  b_tempD += D(b_temp) * isc;
  D b_rhogD = b_rhog;
  if constexpr (kMixed) {
    // pre = (densR pq) temp, pq = qd RDRY + qn0 RVAP, qd = 1 - sum qn (FP32)
    const R tR = R(temp);
    b_tempD = fma(D(b_pre * dpR), isc, b_tempD);
    const R b_dp = b_pre * tR;
    b_densD = fma(D(b_dp * pqR), isc, b_densD);
    const R b_pq = b_dp * densR;
    const D b_qd = D(b_pq * R(RDRY)) * isc;
    b_qn[0] = fma(D(b_pq * R(RVAP)), isc, b_qn[0]);
#pragma unroll
    for (int n = 1; n <= 5; ++n) b_qn[n] -= b_qd;
    // rhoge0 = (temp rhog) CVdry
    const D b_trh = b_rhoge0 * CVDRY;
    b_tempD = fma(b_trh, rhog, b_tempD);
    b_rhogD = fma(b_trh, temp, b_rhogD);
  } else {
    const D b_preD = D(b_pre) * isc;
    b_tempD = fma(b_preD, dp, b_tempD);
    const D b_dp = b_preD * temp;
    b_densD = fma(b_dp, pq, b_densD);
    const D b_pq = b_dp * dens;
    D b_qd = b_pq * RDRY;
    b_qn[0] = fma(b_pq, RVAP, b_qn[0]);
    // rhoge0 = (temp rhog) cv
    const D b_trh = b_rhoge0 * cv;
    const D b_cv = b_rhoge0 * trh;
    b_tempD = fma(b_trh, rhog, b_tempD);
    b_rhogD = fma(b_trh, temp, b_rhogD);
    b_qd = fma(b_cv, CVDRY, b_qd);
#pragma unroll
    for (int n = 1; n <= 5; ++n) b_qn[n] += b_cv * CVDRY - b_qd;
  }
  // qn[n] = rq[n] / rhog (n >= 1); dens = rhog / gsgam2 (mixed: in FP32, the same partials)
  {
#pragma unroll
    for (int n = 1; n <= 5; ++n) {
      b_rq[n] = fma(b_qn[n], rrhog, b_rq[n]);
      b_rhogD = fma(-(b_qn[n] * qn[n]), rrhog, b_rhogD);
    }
    const D rgs = 1.0 / in.gsgam2;
    b_rhogD = fma(b_densD, rgs, b_rhogD);
    ib.gsgam2 = fma(-b_densD * dens, rgs, ib.gsgam2);
  }
  // rhog = in.rhog (1 - d2); negative filter
  {
    ib.rhog = fma(b_rhogD, omd, ib.rhog);
    const D b_d2 = -b_rhogD * in.rhog;
    // d2 = rq0a - clip(rq0a): d d2 / d rq0a = clip ? 1 : 0; rq[0] = clip(rq0a)
    const D b_rq0a = (clip[0] ? b_d2 : 0.0) + (clip[0] ? 0.0 : b_rq[0]);
    // rq0a = rq_in0 + diffq; diffq = sum_{clipped} rq_in[n]
    ib.rhogq[0] += b_rq0a;
#pragma unroll
    for (int n = 2; n <= 5; ++n) ib.rhogq[n] += (clip[n] ? b_rq0a : 0.0) + (clip[n] ? 0.0 : b_rq[n]);
    ib.rhogq[1] += b_rq[1];
  }
  ib.tem += b_tempD;
  ib.q0 += b_qn[0];
  // parameters (their adjoints scaled back as above); in the mixed step each
  // cell's contribution is formed in FP32 and accumulated in FP64
  if constexpr (kMixed) {
    const R p2 = (b_K_vtr * C.K_vtr + b_K_raci * C.K_raci + b_K_iacr * C.K_iacr) / C.Cr + b_Cr;
    const R p3 = (b_K_vts * C.K_vts + b_K_sacw * C.K_sacw + b_K_saci * C.K_saci + b_K_vents2 * R(0.5) * C.K_vents2) /
                 C.Cs;
    const R p4 = (b_K_vtg * C.K_vtg + b_K_gacw * C.K_gacw) / C.Cg + b_Cg;
    const R p6 = b_K_aut * C.K_aut / C.kk_aut;
    pb[0] += D(b_beta) * isc;
    pb[1] += D(b_qicrt) * isc;
    pb[2] += D(p2) * isc;
    pb[3] += D(p3) * isc;
    pb[4] += D(p4) * isc;
    pb[5] += D(b_icenuc) * isc;
    pb[6] += D(p6) * isc;
    return;
  }
  pb[0] += D(b_beta) * isc;
  pb[1] += D(b_qicrt) * isc;
  pb[2] += ((D(b_K_vtr) * D(C.K_vtr) + D(b_K_raci) * D(C.K_raci) + D(b_K_iacr) * D(C.K_iacr)) * (1.0 / D(C.Cr)) +
            D(b_Cr)) * isc;
  pb[3] += (D(b_K_vts) * D(C.K_vts) + D(b_K_sacw) * D(C.K_sacw) + D(b_K_saci) * D(C.K_saci) +
            D(b_K_vents2) * 0.5 * D(C.K_vents2)) *
           (1.0 / D(C.Cs)) * isc;
  pb[4] += ((D(b_K_vtg) * D(C.K_vtg) + D(b_K_gacw) * D(C.K_gacw)) * (1.0 / D(C.Cg)) + D(b_Cg)) * isc;
  pb[5] += D(b_icenuc) * isc;
  pb[6] += D(b_K_aut) * D(C.K_aut) / D(C.kk_aut) * isc;
}

#undef NSW6_CK

}  // namespace nsw6
