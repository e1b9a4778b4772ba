// Hand-written adjoint of the per-cell NSW6 physics (nsw6_cell, FP64, the
// reference configuration).
//
// One call recomputes the cell's forward values exactly as nsw6_cell does
// (same operations, same branches) and then runs the reverse sweep statement
// by statement, from the outputs' adjoints back to the inputs' and the seven
// parameters'.  Nothing is recorded: the values the sweep needs stay in the
// thread's registers (and its local memory), so the cost is arithmetic, where
// a recorded tape costs about 32 bytes of memory traffic per operation.
//
// The derivative of every elementary operation is the one the recording
// adjoint (nsw6_ad.cuh, RVar) takes: quotients, products, sums and fused
// multiply-adds by their partials; min / max / select and every branch follow
// the values; exp, log and pow by their closed forms at the table-driven
// values.  Both adjoints are compared on every cell by the GPU tests.
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
__device__ __forceinline__ void bmin(double a, double b, double g, double& ba, double& bb) {
  if (b < a) bb += g;
  else ba += g;
}
__device__ __forceinline__ void bmax(double a, double b, double g, double& ba, double& bb) {
  if (a < b) bb += g;
  else ba += g;
}
__device__ __forceinline__ double bsqrt(double s) { return s > 0.0 ? 0.5 / s : 0.0; }

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
// Slot s of this cell's checkpoint at p[s * stride].
struct CellCk {
  double* p;
  size_t stride;
};
template <int MODE>
__device__ __forceinline__ double ck_keep(const CellCk& ck, int s, double v) {
  if constexpr (MODE == CA_SAVE) ck.p[(size_t)s * ck.stride] = v;
  return v;
}
// The value of expr (not evaluated under CA_LOAD) at slot s.
#define NSW6_CK(s, expr) ((MODE == CA_LOAD) ? ck.p[(size_t)(s) * ck.stride] : ck_keep<MODE>(ck, (s), (expr)))

template <int MODE = CA_FULL>
__device__ __forceinline__ void nsw6_cell_adjoint(const Consts& C, const FastMath& mth, double dt, double rdt,
                                                  const CellIn& in, const CellBar& ob, CellInBar& ib, double* pb,
                                                  CellCk ck = {nullptr, 0}, CellOut* out = nullptr) {
  const double Z = 0.0, ONE = 1.0;
  // ==================================================================== forward
  // ---- negative_filter, mod_mp_nsw6.cpp:1770-1831
  double rq[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] = in.rhogq[n];
  bool clip[6] = {false, false, false, false, false, false};
  double diffq = 0.0;
#pragma unroll
  for (int n = 2; n <= 5; ++n) {
    diffq += rq[n];
    clip[n] = rq[n] < 0.0;
    rq[n] = clip[n] ? 0.0 : rq[n];
  }
#pragma unroll
  for (int n = 2; n <= 5; ++n) diffq -= rq[n];
  rq[0] += diffq;
  double d2 = rq[0];
  clip[0] = rq[0] < 0.0;
  rq[0] = clip[0] ? 0.0 : rq[0];
  d2 -= rq[0];
  const double omd = 1.0 - d2;
  const double rhog = in.rhog * omd;
  const double rrhog = NSW6_CK(0, 1.0 / rhog);
  const double dens = NSW6_CK(1, rhog / in.gsgam2);
  double qn[6];
  qn[0] = in.q0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qn[n] = div_rn(rq[n], rhog, rrhog);
  double qd = 1.0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qd = qd - qn[n];
  double cv = qd * CVDRY;
#pragma unroll
  for (int n = 1; n <= 5; ++n) cv = cv + qn[n] * CVDRY;
  const double temp = in.tem;
  const double trh = temp * rhog;
  const double rhoge0 = trh * cv;
  const double pq = qd * RDRY + qn[0] * RVAP;
  const double dp = dens * pq;
  const double pre = dp * temp;

  // ---- psat / qsat
  const double tmx = dmax(temp, TEM_MIN);
  const double rtem = NSW6_CK(2, 1.0 / tmx);
  const double al = C.LovR_liq * (C.RTEM00 - rtem);
  const double ai = C.LovR_ice * (C.RTEM00 - rtem);
  const double el = NSW6_CK(3, mth.exp(al)), ei = NSW6_CK(4, mth.exp(ai));
  const double psatl = PSAT0 * el;
  const double psati = PSAT0 * ei;
  const double drv = dens * RVAP;
  const double drt = drv * temp;
  const double rdrt = NSW6_CK(5, 1.0 / drt);
  const double qsatl = psatl * rdrt;
  const double qsati = psati * rdrt;

  // ---- TagBigLoop
  const double qv = dmax(qn[0], Z), qc = dmax(qn[1], Z), qr = dmax(qn[2], Z);
  const double qi = dmax(qn[3], Z), qs = dmax(qn[4], Z), qg = dmax(qn[5], Z);
  const double sld = dmax(qsatl, EPS), sid = dmax(qsati, EPS);
  const double Sliq = NSW6_CK(6, qv / sld);
  const double Sice = NSW6_CK(7, qv / sid);
  const double Rdens = NSW6_CK(8, ONE / dens);
  const double rfa = DENS00 * Rdens;
  const double rho_fact = NSW6_CK(9, sqrt(rfa));
  const double temc = temp - TEM00;
  const bool warm = !(temc < Z);
  const bool d1 = (qr >= 1.0E-4);
  const bool d2b = (1.0E-4 >= qr && 1.0E-4 >= qs);
  const bool sps = (Sice >= ONE);
  const double dqv_dt = div_rn(qv, dt, rdt), dqc_dt = div_rn(qc, dt, rdt), dqr_dt = div_rn(qr, dt, rdt);
  const double dqi_dt = div_rn(qi, dt, rdt), dqs_dt = div_rn(qs, dt, rdt), dqg_dt = div_rn(qg, dt, rdt);

  // rain slope parameter
  const bool rain = (qr >= 1.0E-12);
  double r_a = Z, r_b = Z;   // dens qr, (dens qr) K_rlmdr
  double r_s1 = Z;           // sqrt(r_b)
  double RLMDr = Z, RLMDr_dr = Z, RLMDr_2 = Z, RLMDr_3 = Z, RLMDr_1br = Z, RLMDr_2br = Z, RLMDr_3br = Z, RLMDr_7 = Z;
  double RLMDr_3dr = Z, RLMDr_5dr = Z, RLMDr_6dr = Z;
  if (rain) {
    r_a = dens * qr;
    r_b = r_a * C.K_rlmdr;
    r_s1 = NSW6_CK(10, sqrt(r_b));
    RLMDr = NSW6_CK(11, sqrt(r_s1));
    RLMDr_dr = NSW6_CK(12, sqrt(RLMDr));
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
  const double xs_a = dens * qs;
  const double Xs2 = xs_a * C.rAs;
  const bool snow = (Xs2 >= 1.0E-12);
  double mom[7] = {Z, Z, Z, Z, Z, Z, Z};
  double mlb[7] = {Z, Z, Z, Z, Z, Z, Z};   // b of each moment (d mom / d logX = mom b)
  double RMOMs_Vt = Z, logX = Z;
  double tems = Z;
  bool tems_sel = false;   // tems = temc (else the constant -0.1)
  if (snow) {
    tems_sel = temc < -0.1;   // dmin(-0.1, temc) is temc
    tems = tems_sel ? temc : -0.1;
    logX = NSW6_CK(13, mth.log(Xs2));
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const double* a = C.roh_a + 4 * i;
      const double* b = C.roh_b + 4 * i;
      const double la = __fma_rn(__fma_rn(__fma_rn(a[3], tems, a[2]), tems, a[1]), tems, a[0]);
      const double lb = __fma_rn(__fma_rn(__fma_rn(b[3], tems, b[2]), tems, b[1]), tems, b[0]);
      mlb[i] = lb;
      mom[i] = NSW6_CK(14 + i, mth.exp(__fma_rn(logX, lb, la)));
    }
    RMOMs_Vt = NSW6_CK(21, mom[5] / mom[2]);
  }
  const double MOMs_0 = mom[0], MOMs_1 = mom[1], MOMs_2 = Xs2;
  const double MOMs_0bs = mom[2], MOMs_1bs = mom[3], MOMs_2bs = mom[4], MOMs_2ds = mom[5];
  const double MOMs_5ds_h = mom[6];

  // graupel slope parameter
  const bool graupel = (qg >= 1.0E-12);
  double g_a = Z, g_b = Z, g_s1 = Z;
  double RLMDg = Z, RLMDg_dg = Z, RLMDg_2 = Z, RLMDg_3 = Z, RLMDg_3dg = Z, RLMDg_5dg = Z, g32 = Z;
  if (graupel) {
    g_a = dens * qg;
    g_b = g_a * C.K_rlmdg;
    g_s1 = NSW6_CK(22, sqrt(g_b));
    RLMDg = NSW6_CK(23, sqrt(g_s1));
    RLMDg_dg = NSW6_CK(24, sqrt(RLMDg));
    RLMDg_2 = RLMDg * RLMDg;
    RLMDg_3 = RLMDg_2 * RLMDg;
    RLMDg_3dg = RLMDg_3 * RLMDg_dg;
    g32 = RLMDg_3 * RLMDg_2;
    RLMDg_5dg = g32 * RLMDg_dg;
  }

  // terminal velocity
  const double vtr_a = C.K_vtr * rho_fact;
  const double Vtr = vtr_a * RLMDr_dr;
  const double vts_a = C.K_vts * rho_fact;
  const double Vts = vts_a * RMOMs_Vt;
  const double vtg_a = C.K_vtg * rho_fact;
  const double Vtg = vtg_a * RLMDg_dg;

  // nucleation
  const double nm01 = -0.1 * temc;
  const double nmax = dmax(nm01, Z);
  const double nex = 1.33 * (C.ln1000 + nmax);
  const double nexp = NSW6_CK(25, mth.exp(nex));
  const double qi0a = C.ice_nuc * nexp;
  const double Qi0 = qi0a * Rdens;
  const double pg1 = Qi0 - qi, pg2 = qv - qsati;
  const double pgmin = dmin(pg1, pg2);
  const double pgmax = dmax(pgmin, Z);
  double Pigen = pgmax * rdt;

  // accretion
  double Esi_mod = C.Esi, betai = C.beta_saut, eg = Z;
  bool esi_exp = false, bet_exp = false;   // Esi_mod / betai took the exponential branch of min
  const bool cold_branch = !(warm && C.Esi >= Z && C.beta_saut >= Z);
  if (cold_branch) {
    eg = NSW6_CK(26, mth.exp(C.gamma_sacr * temc));
    const double es = C.Esi * eg;
    esi_exp = es < C.Esi;
    Esi_mod = esi_exp ? es : C.Esi;
    const double bs = C.beta_saut * eg;   // gamma_saut == gamma_sacr
    bet_exp = bs < C.beta_saut;
    betai = bet_exp ? bs : C.beta_saut;
  }
  const double qcqr = qc * qr;
  double Pracw = Z, prw_pow = Z;
  const bool prw_on = (qcqr >= 1.0E-12);
  if (prw_on) {
    prw_pow = NSW6_CK(27, mth.pow(qcqr, 1.15));
    Pracw = 67.0 * prw_pow;
  }
  const double fr = rho_fact;
  const double sacw_a = qc * C.K_sacw, sacw_b = sacw_a * MOMs_2ds;
  double Psacw = sacw_b * fr;
  const double gacw_a = qc * C.K_gacw, gacw_b = gacw_a * RLMDg_3dg;
  double Pgacw = gacw_b * fr;
  const double raci_a = qi * C.K_raci, raci_b = raci_a * RLMDr_3dr;
  double Praci = raci_b * fr;
  const double saci_a = qi * C.K_saci, saci_b = saci_a * Esi_mod, saci_c = saci_b * MOMs_2ds;
  double Psaci = saci_c * fr;
  const double iacr_a = qi * C.K_iacr, iacr_b = iacr_a * RLMDr_6dr;
  double Piacr = iacr_b * fr;
  const double dvrs_d = Vtr - Vts;
  const double dvrs = fabs(dvrs_d);
  const double sacr_k = C.K_sacr * Rdens, sacr_kd = sacr_k * dvrs;
  const double sacr_t1 = C.GAM_1br * RLMDr_1br, sacr_t1m = sacr_t1 * MOMs_2;
  const double sacr_t2 = C.K_2gam2br * RLMDr_2br, sacr_t2m = sacr_t2 * MOMs_1;
  const double sacr_t3 = C.GAM_3br * RLMDr_3br, sacr_t3m = sacr_t3 * MOMs_0;
  const double sacr_s = sacr_t1m + sacr_t2m + sacr_t3m;
  double Psacr = sacr_kd * sacr_s;
  const double dvgr_d = Vtg - Vtr;
  const double dvgr = fabs(dvgr_d);
  const double gacr_k = C.K_gacr * Rdens, gacr_kd = gacr_k * dvgr;
  const double gacr_t1 = C.K_g13 * RLMDr_1br, gacr_t1m = gacr_t1 * RLMDg_3;
  const double gacr_t2 = C.K_g22 * RLMDr_2br, gacr_t2m = gacr_t2 * RLMDg_2;
  const double gacr_t3 = C.GAM_3br * RLMDr_3br, gacr_t3m = gacr_t3 * RLMDg;
  const double gacr_s = gacr_t1m + gacr_t2m + gacr_t3m;
  double Pgacr = gacr_kd * gacr_s;
  const double racs_k = C.K_racs * Rdens, racs_kd = racs_k * dvrs;
  const double racs_t1 = 2.0 * MOMs_0bs, racs_t1m = racs_t1 * RLMDr_3;
  const double racs_t2 = 2.0 * MOMs_1bs, racs_t2m = racs_t2 * RLMDr_2;
  const double racs_t3m = MOMs_2bs * RLMDr;
  const double racs_s = racs_t1m + racs_t2m + racs_t3m;
  double Pracs = racs_kd * racs_s;

  // autoconversion
  const double rhoqc_a = dens * qc;
  const double rhoqc = rhoqc_a * 1000.0;
  double Praut = Z, aut_pow = Z;
  const bool aut_on = qc > Z;
  if (aut_on) {
    aut_pow = NSW6_CK(28, mth.pow(qc, 2.47));
    Praut = C.K_aut * aut_pow;
  }
  const double saut_a = qi - C.qicrt_saut;
  const double saut_b = betai * saut_a;
  double Psaut = dmax(saut_b, Z);

  // evaporation, sublimation, melting and freezing
  const double Ka = (2.428E-2 + 7.47E-5 * temc);
  const double kd0 = (2.222E-5 + 1.37E-7 * temc);
  const double kd1 = kd0 * PSTD;
  const double kd2 = NSW6_CK(29, kd1 / pre);
  const double KdD = kd2 * dens;
  const double nu0 = (1.718E-5 + 5.28E-8 * temc);
  const double rNu = NSW6_CK(30, dens / nu0);
  const double kat = Ka * temp;
  const double rKaT = NSW6_CK(31, ONE / kat);
  const double xi = KdD * qsati;
  const double gv1 = LHS0 * rKaT;
  const double gv2 = C.LovR_ice * rtem;
  const double gv3 = gv2 - ONE;
  const double gv4 = gv1 * gv3;
  const double gv5 = gv4 * xi;
  const double gv6 = gv5 + ONE;
  const double Giv = NSW6_CK(32, xi / gv6);
  const double gil_a = Ka * temc;
  const double Gil = gil_a * C.rLHF0;
  double Prevp = Z;
  double xl = Z, gl1 = Z, gl2 = Z, gl3 = Z, gl4 = Z, gl5 = Z, gl6 = Z, Glv = Z;
  double vr1 = Z, vr2 = Z, vr3 = Z, vr4 = Z, vr5 = Z, vr6 = Z, ventr = Z;
  double ev1 = Z, ev2 = Z, ev3 = Z, ev4 = Z;
  bool sl_min = false;
  if (rain) {
    xl = KdD * qsatl;
    gl1 = LHV0 * rKaT;
    gl2 = C.LovR_liq * rtem;
    gl3 = gl2 - ONE;
    gl4 = gl1 * gl3;
    gl5 = gl4 * xl;
    gl6 = gl5 + ONE;
    Glv = NSW6_CK(33, xl / gl6);
    vr1 = C.K_ventr1 * RLMDr_2;
    vr2 = C.Cr * fr;
    vr3 = vr2 * rNu;
    vr4 = vr3 * RLMDr_5dr;
    vr5 = NSW6_CK(34, sqrt(vr4));
    vr6 = C.K_ventr2 * vr5;
    ventr = vr1 + vr6;
    ev1 = C.K_revp * Rdens;
    sl_min = !(ONE < Sliq);   // dmin(Sliq, 1) = Sliq when !(1 < Sliq)
    ev2 = ONE - (sl_min ? Sliq : ONE);
    ev3 = ev1 * ev2;
    ev4 = ev3 * Glv;
    Prevp = ev4 * ventr;
  }
  const double rhoqi_a = dens * qi;
  const bool rqi_on = !(rhoqi_a < EPS);   // dmax(dens qi, EPS) = dens qi
  const double rhoqi = rqi_on ? rhoqi_a : EPS;
  double XNi = C.XNi_eps, Di = C.Di_eps;
  double xn_pow = Z, xn_a = Z, XMi = Z, di_s = Z, di_a = Z;
  bool xn_lo = false, xn_hi = false, di_cap = false;
  const bool ice_on = rhoqi > EPS;
  if (ice_on) {
    xn_pow = NSW6_CK(35, mth.pow(rhoqi, 0.75));
    xn_a = 5.38E+7 * xn_pow;
    xn_lo = xn_a < 1.0E+3;             // dmax(xn_a, 1e3) gives 1e3
    const double xm = xn_lo ? 1.0E+3 : xn_a;
    xn_hi = 1.0E+6 < xm;               // dmin(xm, 1e6) gives 1e6
    XNi = xn_hi ? 1.0E+6 : xm;
    XMi = NSW6_CK(36, rhoqi / XNi);
    di_s = NSW6_CK(37, sqrt(XMi));
    di_a = C.Di_a * di_s;
    di_cap = C.Di_max < di_a;
    Di = di_cap ? C.Di_max : di_a;
  }
  const double t1a = 4.0 * Di, t1b = t1a * XNi, t1c = t1b * Rdens, sm1 = Sice - ONE, t1d = t1c * sm1;
  const double tmp1 = t1d * Giv;
  double Pidep = sel(sps, tmp1);
  double Pisub = sel(!sps, -tmp1);
  const bool below40 = (temc + 40.0 < Z);
  double Pihom = below40 ? dqc_dt : Z;
  const double efa = -C.A_frz * temc;
  const double efe = NSW6_CK(38, mth.exp(efa));
  const double efrz = efe - ONE;
  const bool htr_on = (!below40 && !warm);
  const double qc2 = qc * qc;
  const double ht1 = dens * qc2, ht2 = ht1 * C.K_ihtr;
  double Pihtr = htr_on ? ht2 * efrz : Z;
  double Pimlt = warm ? dqi_dt : Z;
  const double vs1 = 0.65 * MOMs_1;
  const double vs2 = fr * rNu;
  const double vs3 = NSW6_CK(39, sqrt(vs2));
  const double vs4 = C.K_vents2 * vs3;
  const double vs5 = vs4 * MOMs_5ds_h;
  const double vents = vs1 + vs5;
  const double s1a = C.K_2pi * Rdens, s1b = s1a * sm1, s1c = s1b * Giv;
  const double tmp2 = s1c * vents;
  double Psdep = sel(sps, tmp2);
  double Pssub = sel(!sps, -tmp2);
  const double sm_a = s1a * Gil, sm_b = sm_a * vents;
  const double sm_c = C.K_clf * temc, sm_d = Psacw + Psacr, sm_e = sm_c * sm_d;
  const double sm_f = sm_b + sm_e;
  double Psmlt = dmax(sm_f, Z);
  const double vg1 = C.K_ventg1 * RLMDg_2;
  const double vg2 = C.Cg * fr, vg3 = vg2 * rNu, vg4 = vg3 * RLMDg_5dg;
  const double vg5 = NSW6_CK(40, sqrt(vg4));
  const double vg6 = C.K_ventg2 * vg5;
  const double ventg = vg1 + vg6;
  const double g1a = C.K_gdep * Rdens, g1b = g1a * sm1, g1c = g1b * Giv;
  const double tmp3 = g1c * ventg;
  double Pgdep = sel(sps, tmp3);
  double Pgsub = sel(!sps, -tmp3);
  const double gm_a = g1a * Gil, gm_b = gm_a * ventg;
  const double gm_d = Pgacw + Pgacr, gm_e = sm_c * gm_d;
  const double gm_f = gm_b + gm_e;
  double Pgmlt = dmax(gm_f, Z);
  const double gf_a = C.K_gfrz * Rdens, gf_b = gf_a * efrz;
  double Pgfrz = gf_b * RLMDr_7;

  // limiters (:1249-1296); each records which operand of min it took
  const bool cold = !warm;
  const double Pigen0 = Pigen, Pidep0 = Pidep, Psdep0 = Psdep, Pgdep0 = Pgdep;
  Pigen = sel(cold, dmin(Pigen, dqv_dt));
  Pidep = sel(cold, dmin(Pidep, dqv_dt));
  Psdep = sel(cold, dmin(Psdep, dqv_dt));
  Pgdep = sel(cold, dmin(Pgdep, dqv_dt));
  const double Pracw_a = Pracw + sel(warm, Psacw);
  const double Pracw_b = Pracw_a + sel(warm, Pgacw);
  const double Praut0 = Praut, Pracw0 = Pracw_b, Pihom0 = Pihom, Pihtr0 = Pihtr, Psacw0 = Psacw, Pgacw0 = Pgacw;
  Praut = dmin(Praut, dqc_dt);
  Pracw = dmin(Pracw_b, dqc_dt);
  Pihom = sel(cold, dmin(Pihom, dqc_dt));
  Pihtr = sel(cold, dmin(Pihtr, dqc_dt));
  Psacw = sel(cold, dmin(Psacw, dqc_dt));
  Pgacw = sel(cold, dmin(Pgacw, dqc_dt));
  const double Prevp0 = Prevp, Piacr0 = Piacr, Psacr0 = Psacr, Pgacr0 = Pgacr, Pgfrz0 = Pgfrz;
  Prevp = dmin(Prevp, dqr_dt);
  Piacr = sel(cold, dmin(Piacr, dqr_dt));
  Psacr = sel(cold, dmin(Psacr, dqr_dt));
  Pgacr = sel(cold, dmin(Pgacr, dqr_dt));
  Pgfrz = sel(cold, dmin(Pgfrz, dqr_dt));
  const double Pisub0 = Pisub, Pimlt0 = Pimlt, Psaut0 = Psaut, Praci0 = Praci, Psaci0 = Psaci;
  Pisub = sel(cold, dmin(Pisub, dqi_dt));
  Pimlt = sel(warm, dmin(Pimlt, dqi_dt));
  Psaut = sel(cold, dmin(Psaut, dqi_dt));
  Praci = sel(cold, dmin(Praci, dqi_dt));
  Psaci = sel(cold, dmin(Psaci, dqi_dt));
  const double Pssub0 = Pssub, Psmlt0 = Psmlt, Pracs0 = Pracs;
  Pssub = sel(cold, dmin(Pssub, dqs_dt));
  Psmlt = sel(warm, dmin(Psmlt, dqs_dt));
  Pracs = sel(cold, dmin(Pracs, dqs_dt));
  const double Pgsub0 = Pgsub, Pgmlt0 = Pgmlt;
  Pgsub = sel(cold, dmin(Pgsub, dqg_dt));
  Pgmlt = sel(warm, dmin(Pgmlt, dqg_dt));
  double Piacr_s = sel(!d1, Piacr);
  double Piacr_g = sel(d1, Piacr);
  double Praci_s = sel(!d1, Praci);
  double Praci_g = sel(d1, Praci);
  double Psacr_s = sel(d2b, Psacr);
  double Psacr_g = sel(!d2b, Psacr);
  const double Pracs1 = Pracs;
  Pracs = sel(!d2b, Pracs);

  // loss limiters: fac = 1 when net + EPS >= 0, else min(-dq / net, 1)
  struct Lim {
    double net, fac;
    bool scaled, ratio;   // fac != 1; fac is -dq / net (else 1 from min)
  };
  auto limit = [&](int slot, double net, double dq) {
    Lim L;
    L.net = net;
    if (net + EPS >= Z) {
      L.fac = ONE;
      L.ratio = false;
    } else {
      const double r = NSW6_CK(slot, -dq / net);
      L.ratio = !(ONE < r);
      L.fac = L.ratio ? r : ONE;
    }
    L.scaled = L.fac != ONE;
    return L;
  };
  // [QC]
  const double QC_in[7] = {Pimlt, Praut, Pracw, Pihom, Pihtr, Psacw, Pgacw};
  const Lim Lc = limit(41, +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw, dqc_dt);
  if (Lc.scaled) {
    Pimlt *= Lc.fac; Praut *= Lc.fac; Pracw *= Lc.fac; Pihom *= Lc.fac; Pihtr *= Lc.fac; Psacw *= Lc.fac;
    Pgacw *= Lc.fac;
  }
  // [QI]
  const double QI_in[10] = {Pigen, Pidep, Pihom, Pihtr, Pisub, Pimlt, Psaut, Praci_s, Psaci, Praci_g};
  const Lim Li = limit(42, +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g, dqi_dt);
  if (Li.scaled) {
    Pigen *= Li.fac; Pidep *= Li.fac; Pihom *= Li.fac; Pihtr *= Li.fac; Pisub *= Li.fac; Pimlt *= Li.fac;
    Psaut *= Li.fac; Praci_s *= Li.fac; Psaci *= Li.fac; Praci_g *= Li.fac;
  }
  // [QR]
  const double QR_in[11] = {Praut, Pracw, Psmlt, Pgmlt, Prevp, Piacr_s, Psacr_s, Piacr_g, Psacr_g, Pgacr, Pgfrz};
  const Lim Lr = limit(43, +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz,
                       dqr_dt);
  if (Lr.scaled) {
    Praut *= Lr.fac; Pracw *= Lr.fac; Psmlt *= Lr.fac; Pgmlt *= Lr.fac; Prevp *= Lr.fac; Piacr_s *= Lr.fac;
    Psacr_s *= Lr.fac; Piacr_g *= Lr.fac; Psacr_g *= Lr.fac; Pgacr *= Lr.fac; Pgfrz *= Lr.fac;
  }
  // [QV]
  const double QV_in[8] = {Prevp, Pisub, Pssub, Pgsub, Pigen, Pidep, Psdep, Pgdep};
  const Lim Lv = limit(44, +Prevp + Pisub + Pssub + Pgsub - Pigen - Pidep - Psdep - Pgdep, dqv_dt);
  if (Lv.scaled) {
    Prevp *= Lv.fac; Pisub *= Lv.fac; Pssub *= Lv.fac; Pgsub *= Lv.fac; Pigen *= Lv.fac; Pidep *= Lv.fac;
    Psdep *= Lv.fac; Pgdep *= Lv.fac;
  }
  // [QS]
  const double QS_in[10] = {Psdep, Psacw, Piacr_s, Psacr_s, Psaut, Praci_s, Psaci, Pssub, Psmlt, Pracs};
  const Lim Ls = limit(45, +Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs, dqs_dt);
  if (Ls.scaled) {
    Psdep *= Ls.fac; Psacw *= Ls.fac; Piacr_s *= Ls.fac; Psacr_s *= Ls.fac; Psaut *= Ls.fac; Praci_s *= Ls.fac;
    Psaci *= Ls.fac; Pssub *= Ls.fac; Psmlt *= Ls.fac; Pracs *= Ls.fac;
  }
  // [QG]
  const double QG_in[10] = {Pgdep, Pgacw, Piacr_g, Psacr_g, Pgacr, Pgfrz, Praci_g, Pracs, Pgsub, Pgmlt};
  const Lim Lg = limit(46, +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt, dqg_dt);
  if (Lg.scaled) {
    Pgdep *= Lg.fac; Pgacw *= Lg.fac; Piacr_g *= Lg.fac; Psacr_g *= Lg.fac; Pgacr *= Lg.fac; Pgfrz *= Lg.fac;
    Praci_g *= Lg.fac; Pracs *= Lg.fac; Pgsub *= Lg.fac; Pgmlt *= Lg.fac;
  }

  // tendencies
  const double qc_t0 = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw;
  const double qr_t0 = +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz;
  const double qi_t0 = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g;
  const double qs_t0 = +Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs;
  const double qg_t0 = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt;
  // qx_t = max(qx_t0, -dqx_dt): true when the tendency itself is kept
  const bool kc_ = !(qc_t0 < -dqc_dt), kr_ = !(qr_t0 < -dqr_dt), ki_ = !(qi_t0 < -dqi_dt);
  const bool ks_ = !(qs_t0 < -dqs_dt), kg_ = !(qg_t0 < -dqg_dt);
  const double qc_t = kc_ ? qc_t0 : -dqc_dt, qr_t = kr_ ? qr_t0 : -dqr_dt, qi_t = ki_ ? qi_t0 : -dqi_dt;
  const double qs_t = ks_ ? qs_t0 : -dqs_dt, qg_t = kg_ ? qg_t0 : -dqg_dt;
  const double qv_t = -(qc_t + qr_t + qi_t + qs_t + qg_t);
  const double qt[6] = {qv_t, qc_t, qr_t, qi_t, qs_t, qg_t};
  double rq2[6], rqt[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    rqt[n] = rhog * qt[n];
    rq2[n] = rq[n] + rqt[n] * dt;
  }
  // effective radius and cloud top
  const double xf1 = rhoqc * C.K_xf;
  const double xf2 = C.coef_xf * xf1;
  const double xf3 = xf2 + EPS;
  const double rf_qc = NSW6_CK(47, mth.pow(xf3, 0.33333333));
  const double rf2 = rf_qc * rf_qc;
  const double r2_qc = C.K_r2c * rf2;
  const double r2_qr = C.K_r2r * RLMDr_3;
  const double r3c_a = C.coef_xf * dens, r3_qc = r3c_a * qc;
  const double r3_qr = r3c_a * qr;
  const double r2 = r2_qc + r2_qr;
  const bool big = (r2 >= 1.0E-10);
  const double r3 = r3_qc + r3_qr;
  const bool top = !big && ((qc + qr) >= 1.0E-5);
  const bool cld = (r2_qc >= 1.0E-10);
  // updates
  const double rhoge1 = rhoge0 - LHV0 * (rqt[0] * dt);
  const double rhoge2 = rhoge1 + LHF0 * (rqt[3] * dt);
  const double rhoge3 = rhoge2 + LHF0 * (rqt[4] * dt);
  const double rhoge = rhoge3 + LHF0 * (rqt[5] * dt);
  double q2[6];
  q2[0] = qn[0];
#pragma unroll
  for (int n = 1; n <= 5; ++n) q2[n] = div_rn(rq2[n], rhog, rrhog);
  double qd2 = 1.0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qd2 = qd2 - q2[n];
  double cva = qd2 * CVDRY;
#pragma unroll
  for (int n = 1; n <= 5; ++n) cva = cva + q2[n] * CVDRY;
  const double rcva = rhog * cva;
  const double tem_o = NSW6_CK(48, rhoge / rcva);
  if constexpr (MODE == CA_SAVE) {
    // the outputs of nsw6_cell (the same operations on the same values)
    out->Vtr = Vtr;
    out->Vts = Vts;
    out->Vtg = Vtg;
    out->Vti = 0.0;
    out->rceff = big ? r3 / r2 : Z;
    out->rctop = top ? out->rceff : UNDEF;
    out->tctop = top ? temp : UNDEF;
    out->rceff_cld = cld ? r3_qc / r2_qc : 0.0;
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
  // adjoints of the outputs
  double b_rhog = ob.rhog, b_rhoge = ob.rhoge;
  double b_rq2[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) b_rq2[n] = ob.rhogq[n];
  double b_q2[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) b_q2[n] = ob.q[n];
  // tem_o = rhoge / rcva
  {
    const double g = ob.tem;
    const double rr = 1.0 / rcva;
    b_rhoge = fma(g, rr, b_rhoge);
    const double b_rcva = -g * tem_o * rr;
    b_rhog = fma(b_rcva, cva, b_rhog);
    const double b_cva = b_rcva * rhog;
    // cva = qd2 CV + sum q2 CV
    const double b_qd2 = b_cva * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) b_q2[n] += b_cva * CVDRY - b_qd2;
  }
  // q2[n] = rq2[n] / rhog
#pragma unroll
  for (int n = 1; n <= 5; ++n) {
    b_rq2[n] = fma(b_q2[n], rrhog, b_rq2[n]);
    b_rhog = fma(-(b_q2[n] * q2[n]), rrhog, b_rhog);
  }
  // rhoge = rhoge0 - LHV0 rqt0 dt + LHF0 (rqt3 + rqt4 + rqt5) dt
  double b_rhoge0 = b_rhoge;
  double b_rqt[6] = {0, 0, 0, 0, 0, 0};
  b_rqt[0] = fma(-(b_rhoge * LHV0), dt, b_rqt[0]);
  b_rqt[3] = fma(b_rhoge * LHF0, dt, b_rqt[3]);
  b_rqt[4] = fma(b_rhoge * LHF0, dt, b_rqt[4]);
  b_rqt[5] = fma(b_rhoge * LHF0, dt, b_rqt[5]);
  // rq2 = rq + rqt dt
  double b_rq[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    b_rq[n] = b_rq2[n];
    b_rqt[n] = fma(b_rq2[n], dt, b_rqt[n]);
  }
  // rqt = rhog qt
  double b_qt[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    b_rhog = fma(b_rqt[n], qt[n], b_rhog);
    b_qt[n] = b_rqt[n] * rhog;
  }
  // effective radius and cloud top: adjoints of the dens, qc, qr, RLMDr_3, temp they read
  double b_dens = 0.0, b_qc = 0.0, b_qr = 0.0, b_RLMDr_3 = 0.0, b_temp = 0.0, b_rhoqc = 0.0;
  {
    double b_r2_qc = 0.0, b_r2_qr = 0.0, b_r3_qc = 0.0, b_r3_qr = 0.0;
    // rceff = big ? r3 / r2 : 0
    if (big) {
      const double rr2 = 1.0 / r2;
      const double b_r3 = ob.rceff * rr2;
      const double b_r2 = -ob.rceff * (r3 * rr2) * rr2;
      b_r3_qc += b_r3;
      b_r3_qr += b_r3;
      b_r2_qc += b_r2;
      b_r2_qr += b_r2;
    }
    // rctop = top ? rceff (= 0, !big) : UNDEF; tctop = top ? temp : UNDEF
    if (top) b_temp += ob.tctop;
    // rceff_cld = cld ? r3_qc / r2_qc : 0
    if (cld) {
      const double rr2 = 1.0 / r2_qc;
      b_r3_qc = fma(ob.rceff_cld, rr2, b_r3_qc);
      b_r2_qc = fma(-(ob.rceff_cld * (r3_qc * rr2)), rr2, b_r2_qc);
    }
    // r3_qc = (coef_xf dens) qc, r3_qr = (coef_xf dens) qr
    b_qc = fma(b_r3_qc, r3c_a, b_qc);
    b_qr = fma(b_r3_qr, r3c_a, b_qr);
    b_dens = fma((b_r3_qc * qc + b_r3_qr * qr), C.coef_xf, b_dens);
    // r2_qr = K_r2r RLMDr_3
    b_RLMDr_3 = fma(b_r2_qr, C.K_r2r, b_RLMDr_3);
    // r2_qc = K_r2c rf^2, rf = pow(xf3, 1/3)
    const double b_rf = b_r2_qc * C.K_r2c * 2.0 * rf_qc;
    const double b_xf3 = (xf3 > 0.0) ? b_rf * 0.33333333 * rf_qc / xf3 : 0.0;
    b_rhoqc = fma(b_xf3 * C.coef_xf, C.K_xf, b_rhoqc);
  }
  // Vt outputs
  double b_Vtr = ob.Vtr, b_Vts = ob.Vts, b_Vtg = ob.Vtg;

  // qv_t = -(qc_t + qr_t + qi_t + qs_t + qg_t)
  double b_qc_t = b_qt[1] - b_qt[0], b_qr_t = b_qt[2] - b_qt[0], b_qi_t = b_qt[3] - b_qt[0];
  double b_qs_t = b_qt[4] - b_qt[0], b_qg_t = b_qt[5] - b_qt[0];
  // qx_t = max(qx_t0, -dqx_dt)
  double b_dqv = 0.0, b_dqc = 0.0, b_dqr = 0.0, b_dqi = 0.0, b_dqs = 0.0, b_dqg = 0.0;
  const double b_qc_t0 = kc_ ? b_qc_t : 0.0;
  if (!kc_) b_dqc -= b_qc_t;
  const double b_qr_t0 = kr_ ? b_qr_t : 0.0;
  if (!kr_) b_dqr -= b_qr_t;
  const double b_qi_t0 = ki_ ? b_qi_t : 0.0;
  if (!ki_) b_dqi -= b_qi_t;
  const double b_qs_t0 = ks_ ? b_qs_t : 0.0;
  if (!ks_) b_dqs -= b_qs_t;
  const double b_qg_t0 = kg_ ? b_qg_t : 0.0;
  if (!kg_) b_dqg -= b_qg_t;
  // tendency sums: adjoints of the (limited) rates
  double bPimlt = b_qc_t0 - b_qi_t0, bPraut = -b_qc_t0 + b_qr_t0, bPracw = -b_qc_t0 + b_qr_t0;
  double bPihom = -b_qc_t0 + b_qi_t0, bPihtr = -b_qc_t0 + b_qi_t0, bPsacw = -b_qc_t0 + b_qs_t0;
  double bPgacw = -b_qc_t0 + b_qg_t0;
  double bPsmlt = b_qr_t0 - b_qs_t0, bPgmlt = b_qr_t0 - b_qg_t0, bPrevp = -b_qr_t0;
  double bPiacr_s = -b_qr_t0 + b_qs_t0, bPsacr_s = -b_qr_t0 + b_qs_t0, bPiacr_g = -b_qr_t0 + b_qg_t0;
  double bPsacr_g = -b_qr_t0 + b_qg_t0, bPgacr = -b_qr_t0 + b_qg_t0, bPgfrz = -b_qr_t0 + b_qg_t0;
  double bPigen = b_qi_t0, bPidep = b_qi_t0, bPisub = -b_qi_t0, bPsaut = -b_qi_t0 + b_qs_t0;
  double bPraci_s = -b_qi_t0 + b_qs_t0, bPsaci = -b_qi_t0 + b_qs_t0, bPraci_g = -b_qi_t0 + b_qg_t0;
  double bPsdep = b_qs_t0, bPssub = -b_qs_t0, bPracs = -b_qs_t0 + b_qg_t0;
  double bPgdep = b_qg_t0, bPgsub = -b_qg_t0;

  // loss limiters in reverse: x_out = x_in * fac, fac = min(-dq / net, 1), net = sum(+-x_in)
  auto unlimit = [&](const Lim& L, double* const* bx, const double* xin, const double* sgn, int n, double dq,
                     double& b_dq) {
    if (!L.scaled) return;
    double b_fac = 0.0;
    for (int j = 0; j < n; ++j) {
      b_fac = fma(*bx[j], xin[j], b_fac);
      *bx[j] *= L.fac;
    }
    if (L.ratio) {   // fac = -dq / net
      const double rnet = 1.0 / L.net;
      b_dq = fma(-b_fac, rnet, b_dq);
      const double b_net = b_fac * dq * (rnet * rnet);
      for (int j = 0; j < n; ++j) *bx[j] += sgn[j] * b_net;
    }
  };
  {  // [QG]
    double* bx[10] = {&bPgdep, &bPgacw, &bPiacr_g, &bPsacr_g, &bPgacr, &bPgfrz, &bPraci_g, &bPracs, &bPgsub, &bPgmlt};
    const double sg[10] = {1, 1, 1, 1, 1, 1, 1, 1, -1, -1};
    unlimit(Lg, bx, QG_in, sg, 10, dqg_dt, b_dqg);
  }
  {  // [QS]
    double* bx[10] = {&bPsdep, &bPsacw, &bPiacr_s, &bPsacr_s, &bPsaut, &bPraci_s, &bPsaci, &bPssub, &bPsmlt, &bPracs};
    const double sg[10] = {1, 1, 1, 1, 1, 1, 1, -1, -1, -1};
    unlimit(Ls, bx, QS_in, sg, 10, dqs_dt, b_dqs);
  }
  {  // [QV]
    double* bx[8] = {&bPrevp, &bPisub, &bPssub, &bPgsub, &bPigen, &bPidep, &bPsdep, &bPgdep};
    const double sg[8] = {1, 1, 1, 1, -1, -1, -1, -1};
    unlimit(Lv, bx, QV_in, sg, 8, dqv_dt, b_dqv);
  }
  {  // [QR]
    double* bx[11] = {&bPraut, &bPracw, &bPsmlt, &bPgmlt, &bPrevp, &bPiacr_s, &bPsacr_s, &bPiacr_g, &bPsacr_g,
                      &bPgacr, &bPgfrz};
    const double sg[11] = {1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1};
    unlimit(Lr, bx, QR_in, sg, 11, dqr_dt, b_dqr);
  }
  {  // [QI]
    double* bx[10] = {&bPigen, &bPidep, &bPihom, &bPihtr, &bPisub, &bPimlt, &bPsaut, &bPraci_s, &bPsaci, &bPraci_g};
    const double sg[10] = {1, 1, 1, 1, -1, -1, -1, -1, -1, -1};
    unlimit(Li, bx, QI_in, sg, 10, dqi_dt, b_dqi);
  }
  {  // [QC]
    double* bx[7] = {&bPimlt, &bPraut, &bPracw, &bPihom, &bPihtr, &bPsacw, &bPgacw};
    const double sg[7] = {1, -1, -1, -1, -1, -1, -1};
    unlimit(Lc, bx, QC_in, sg, 7, dqc_dt, b_dqc);
  }
  // species splits
  if (d2b) bPracs = 0.0;   // Pracs = sel(!d2b, Pracs1)
  double bPsacr = (d2b ? bPsacr_s : 0.0) + (!d2b ? bPsacr_g : 0.0);
  double bPraci = (!d1 ? bPraci_s : 0.0) + (d1 ? bPraci_g : 0.0);
  double bPiacr = (!d1 ? bPiacr_s : 0.0) + (d1 ? bPiacr_g : 0.0);
  (void)Pracs1;
  // limiters in reverse: x = sel(on, min(x0, dq))
  auto unmin = [&](bool on, double x0, double dq, double& bx, double& b_dq) {
    if (!on) {
      bx = 0.0;
      return;
    }
    const double g = bx;
    bx = 0.0;
    bmin(x0, dq, g, bx, b_dq);
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
  double bPracw0 = bPracw;
  double bPsacw_w = warm ? bPracw : 0.0, bPgacw_w = warm ? bPracw : 0.0;
  bPsacw += bPsacw_w;
  bPgacw += bPgacw_w;
  unmin(cold, Pgdep0, dqv_dt, bPgdep, b_dqv);
  unmin(cold, Psdep0, dqv_dt, bPsdep, b_dqv);
  unmin(cold, Pidep0, dqv_dt, bPidep, b_dqv);
  unmin(cold, Pigen0, dqv_dt, bPigen, b_dqv);

  // ---- process rates in reverse
  double b_rho_fact = 0.0, b_Rdens = 0.0, b_temc = 0.0, b_rNu = 0.0, b_Giv = 0.0, b_Gil = 0.0, b_Sice = 0.0;
  double b_Sliq = 0.0, b_qv = 0.0, b_qi = 0.0, b_qs = 0.0, b_qg = 0.0, b_qsati = 0.0, b_qsatl = 0.0;
  double b_RLMDr = 0.0, b_RLMDr_dr = 0.0, b_RLMDr_2 = 0.0, b_RLMDr_1br = 0.0, b_RLMDr_2br = 0.0;
  double b_RLMDr_3br = 0.0, b_RLMDr_7 = 0.0, b_RLMDr_3dr = 0.0, b_RLMDr_5dr = 0.0, b_RLMDr_6dr = 0.0;
  double b_RLMDg = 0.0, b_RLMDg_dg = 0.0, b_RLMDg_2 = 0.0, b_RLMDg_3 = 0.0, b_RLMDg_3dg = 0.0, b_RLMDg_5dg = 0.0;
  double b_mom[7] = {0, 0, 0, 0, 0, 0, 0};
  double b_MOMs_2 = 0.0, b_RMOMs_Vt = 0.0, b_Esi_mod = 0.0, b_betai = 0.0, b_efrz = 0.0, b_pre = 0.0, b_rtem = 0.0;
  double b_KdD = 0.0, b_Ka = 0.0, b_Di = 0.0, b_XNi = 0.0, b_rhoqi = 0.0;
  // parameter-dependent constants
  double b_K_vtr = 0.0, b_K_raci = 0.0, b_K_iacr = 0.0, b_Cr = 0.0, b_K_vts = 0.0, b_K_sacw = 0.0, b_K_saci = 0.0;
  double b_K_vents2 = 0.0, b_K_vtg = 0.0, b_K_gacw = 0.0, b_Cg = 0.0, b_beta = 0.0, b_qicrt = 0.0, b_icenuc = 0.0;
  double b_K_aut = 0.0;

  // Pgfrz = (K_gfrz Rdens) efrz RLMDr_7
  b_Rdens = fma(bPgfrz * RLMDr_7 * efrz, C.K_gfrz, b_Rdens);
  b_efrz = fma(bPgfrz * RLMDr_7, gf_a, b_efrz);
  b_RLMDr_7 = fma(bPgfrz, gf_b, b_RLMDr_7);
  // Pgmlt = max(gm_b + sm_c gm_d, 0); gm_b = (g1a Gil) ventg; gm_d = Pgacw + Pgacr
  double b_ventg = 0.0, b_g1a = 0.0, b_sm_c = 0.0;
  {
    double b_f = 0.0, dummy = 0.0;
    bmax(gm_f, Z, bPgmlt, b_f, dummy);
    b_g1a = fma(b_f * ventg, Gil, b_g1a);
    b_Gil = fma(b_f * ventg, g1a, b_Gil);
    b_ventg = fma(b_f, gm_a, b_ventg);
    b_sm_c = fma(b_f, gm_d, b_sm_c);
    bPgacw = fma(b_f, sm_c, bPgacw);
    bPgacr = fma(b_f, sm_c, bPgacr);
  }
  // Pgdep = sel(sps, tmp3), Pgsub = sel(!sps, -tmp3); tmp3 = (g1a sm1 Giv) ventg
  {
    const double b_t = (sps ? bPgdep : 0.0) - (!sps ? bPgsub : 0.0);
    b_g1a = fma(b_t * ventg * Giv, sm1, b_g1a);
    b_Sice = fma(b_t * ventg * Giv, g1a, b_Sice);
    b_Giv = fma(b_t * ventg, g1b, b_Giv);
    b_ventg = fma(b_t, g1c, b_ventg);
  }
  // g1a = K_gdep Rdens
  b_Rdens = fma(b_g1a, C.K_gdep, b_Rdens);
  // ventg = K_ventg1 RLMDg_2 + K_ventg2 sqrt(Cg fr rNu RLMDg_5dg)
  {
    b_RLMDg_2 = fma(b_ventg, C.K_ventg1, b_RLMDg_2);
    const double b_vg5 = b_ventg * C.K_ventg2;
    const double b_vg4 = b_vg5 * bsqrt(vg5);
    b_RLMDg_5dg = fma(b_vg4, vg3, b_RLMDg_5dg);
    const double b_vg3 = b_vg4 * RLMDg_5dg;
    b_rNu = fma(b_vg3, vg2, b_rNu);
    const double b_vg2 = b_vg3 * rNu;
    b_Cg = fma(b_vg2, fr, b_Cg);
    b_rho_fact = fma(b_vg2, C.Cg, b_rho_fact);
  }
  // Psmlt = max(sm_b + sm_c sm_d, 0); sm_b = (s1a Gil) vents; sm_d = Psacw + Psacr
  double b_vents = 0.0, b_s1a = 0.0;
  {
    double b_f = 0.0, dummy = 0.0;
    bmax(sm_f, Z, bPsmlt, b_f, dummy);
    b_s1a = fma(b_f * vents, Gil, b_s1a);
    b_Gil = fma(b_f * vents, s1a, b_Gil);
    b_vents = fma(b_f, sm_a, b_vents);
    b_sm_c = fma(b_f, sm_d, b_sm_c);
    bPsacw = fma(b_f, sm_c, bPsacw);
    bPsacr = fma(b_f, sm_c, bPsacr);
  }
  // sm_c = K_clf temc
  b_temc = fma(b_sm_c, C.K_clf, b_temc);
  // Psdep / Pssub: tmp2 = (s1a sm1 Giv) vents
  {
    const double b_t = (sps ? bPsdep : 0.0) - (!sps ? bPssub : 0.0);
    b_s1a = fma(b_t * vents * Giv, sm1, b_s1a);
    b_Sice = fma(b_t * vents * Giv, s1a, b_Sice);
    b_Giv = fma(b_t * vents, s1b, b_Giv);
    b_vents = fma(b_t, s1c, b_vents);
  }
  b_Rdens = fma(b_s1a, C.K_2pi, b_Rdens);
  // vents = 0.65 MOMs_1 + (K_vents2 sqrt(fr rNu)) MOMs_5ds_h
  {
    b_mom[1] = fma(b_vents, 0.65, b_mom[1]);
    b_mom[6] = fma(b_vents, vs4, b_mom[6]);
    const double b_vs4 = b_vents * MOMs_5ds_h;
    b_K_vents2 = fma(b_vs4, vs3, b_K_vents2);
    const double b_vs2 = b_vs4 * C.K_vents2 * bsqrt(vs3);
    b_rho_fact = fma(b_vs2, rNu, b_rho_fact);
    b_rNu = fma(b_vs2, fr, b_rNu);
  }
  // Pimlt = warm ? dqi_dt : 0
  if (warm) b_dqi += bPimlt;
  // Pihtr = htr_on ? (dens qc^2 K_ihtr) efrz : 0
  if (htr_on) {
    b_efrz = fma(bPihtr, ht2, b_efrz);
    const double b_ht1 = bPihtr * efrz * C.K_ihtr;
    b_dens = fma(b_ht1, qc2, b_dens);
    b_qc = fma(b_ht1 * dens * 2.0, qc, b_qc);
  }
  // efrz = exp(-A_frz temc) - 1
  b_temc = fma(b_efrz * efe, (-C.A_frz), b_temc);
  // Pihom = below40 ? dqc_dt : 0
  if (below40) b_dqc += bPihom;
  // Pidep / Pisub: tmp1 = (((4 Di) XNi) Rdens sm1) Giv
  {
    const double b_t = (sps ? bPidep : 0.0) - (!sps ? bPisub : 0.0);
    b_Giv = fma(b_t, t1d, b_Giv);
    const double b_t1d = b_t * Giv;
    b_Sice = fma(b_t1d, t1c, b_Sice);
    const double b_t1c = b_t1d * sm1;
    b_Rdens = fma(b_t1c, t1b, b_Rdens);
    const double b_t1b = b_t1c * Rdens;
    b_XNi = fma(b_t1b, t1a, b_XNi);
    b_Di = fma(b_t1b * XNi, 4.0, b_Di);
  }
  // XNi, Di from rhoqi
  if (ice_on) {
    if (!di_cap) {
      const double b_dia = b_Di;
      const double b_dis = b_dia * C.Di_a;
      const double b_XMi = b_dis * bsqrt(di_s);
      const double rXNi = 1.0 / XNi;
      b_rhoqi = fma(b_XMi, rXNi, b_rhoqi);
      b_XNi = fma(-(b_XMi * XMi), rXNi, b_XNi);
    }
    // XNi = min(max(5.38e7 pow(rhoqi, 0.75), 1e3), 1e6)
    if (!xn_hi && !xn_lo) {
      const double b_pow = b_XNi * 5.38E+7;
      if (rhoqi > 0.0) b_rhoqi += b_pow * 0.75 * xn_pow / rhoqi;
    }
  }
  if (rqi_on) {
    b_dens = fma(b_rhoqi, qi, b_dens);
    b_qi = fma(b_rhoqi, dens, b_qi);
  }
  // Prevp = (((K_revp Rdens) (1 - min(Sliq, 1))) Glv) ventr
  if (rain) {
    const double b_ventr = bPrevp * ev4;
    const double b_ev4 = bPrevp * ventr;
    const double b_Glv = b_ev4 * ev3;
    const double b_ev3 = b_ev4 * Glv;
    const double b_ev1 = b_ev3 * ev2;
    const double b_ev2 = b_ev3 * ev1;
    if (sl_min) b_Sliq -= b_ev2;
    b_Rdens = fma(b_ev1, C.K_revp, b_Rdens);
    // ventr = K_ventr1 RLMDr_2 + K_ventr2 sqrt(Cr fr rNu RLMDr_5dr)
    b_RLMDr_2 = fma(b_ventr, C.K_ventr1, b_RLMDr_2);
    const double b_vr4 = b_ventr * C.K_ventr2 * bsqrt(vr5);
    b_RLMDr_5dr = fma(b_vr4, vr3, b_RLMDr_5dr);
    const double b_vr3 = b_vr4 * RLMDr_5dr;
    b_rNu = fma(b_vr3, vr2, b_rNu);
    const double b_vr2 = b_vr3 * rNu;
    b_Cr = fma(b_vr2, fr, b_Cr);
    b_rho_fact = fma(b_vr2, C.Cr, b_rho_fact);
    // Glv = xl / (((LHV0 rKaT) (LovR_liq rtem - 1)) xl + 1)
    const double rgl6 = 1.0 / gl6;
    const double b_xl0 = b_Glv * rgl6;
    const double b_gl6 = -b_Glv * Glv * rgl6;
    const double b_gl4 = b_gl6 * xl;
    const double b_xl = b_xl0 + b_gl6 * gl4;
    const double b_gl1 = b_gl4 * gl3;
    const double b_gl3 = b_gl4 * gl1;
    b_rtem = fma(b_gl3, C.LovR_liq, b_rtem);
    const double b_rKaT_l = b_gl1 * LHV0;
    // xl = KdD qsatl
    b_KdD = fma(b_xl, qsatl, b_KdD);
    b_qsatl = fma(b_xl, KdD, b_qsatl);
    // rKaT = 1 / (Ka temp)
    const double b_kat = -b_rKaT_l * rKaT * rKaT;
    b_Ka = fma(b_kat, temp, b_Ka);
    b_temp = fma(b_kat, Ka, b_temp);
  }
  // Gil = (Ka temc) rLHF0
  {
    const double b_gila = b_Gil * C.rLHF0;
    b_Ka = fma(b_gila, temc, b_Ka);
    b_temc = fma(b_gila, Ka, b_temc);
  }
  // Giv = xi / (((LHS0 rKaT) (LovR_ice rtem - 1)) xi + 1)
  {
    const double rgv6 = 1.0 / gv6;
    const double b_xi0 = b_Giv * rgv6;
    const double b_gv6 = -b_Giv * Giv * rgv6;
    const double b_gv4 = b_gv6 * xi;
    const double b_xi = b_xi0 + b_gv6 * gv4;
    const double b_gv1 = b_gv4 * gv3;
    const double b_gv3 = b_gv4 * gv1;
    b_rtem = fma(b_gv3, C.LovR_ice, b_rtem);
    const double b_rKaT = b_gv1 * LHS0;
    const double b_kat = -b_rKaT * rKaT * rKaT;
    b_Ka = fma(b_kat, temp, b_Ka);
    b_temp = fma(b_kat, Ka, b_temp);
    b_KdD = fma(b_xi, qsati, b_KdD);
    b_qsati = fma(b_xi, KdD, b_qsati);
  }
  // rNu = dens / nu0, nu0 = 1.718e-5 + 5.28e-8 temc
  {
    const double rnu0 = 1.0 / nu0;
    b_dens = fma(b_rNu, rnu0, b_dens);
    const double b_nu0 = -b_rNu * rNu * rnu0;
    b_temc = fma(b_nu0, 5.28E-8, b_temc);
  }
  // KdD = ((kd0 PSTD) / pre) dens, kd0 = 2.222e-5 + 1.37e-7 temc
  {
    b_dens = fma(b_KdD, kd2, b_dens);
    const double b_kd2 = b_KdD * dens;
    const double rpre = 1.0 / pre;
    const double b_kd1 = b_kd2 * rpre;
    b_pre = fma(-(b_kd2 * kd2), rpre, b_pre);
    b_temc = fma(b_kd1 * PSTD, 1.37E-7, b_temc);
  }
  // Ka = 2.428e-2 + 7.47e-5 temc
  b_temc = fma(b_Ka, 7.47E-5, b_temc);
  // Psaut = max(betai (qi - qicrt), 0), off where its argument is exactly 0
  // (rate_on: a cell without ice at the threshold qicrt = 0)
  {
    const double b_sb = saut_b > Z ? bPsaut : 0.0;
    b_betai = fma(b_sb, saut_a, b_betai);
    const double b_sa = b_sb * betai;
    b_qi += b_sa;
    b_qicrt -= b_sa;
  }
  // Praut = K_aut pow(qc, 2.47)
  if (aut_on) {
    b_K_aut = fma(bPraut, aut_pow, b_K_aut);
    if (qc > 0.0) b_qc += bPraut * C.K_aut * 2.47 * aut_pow / qc;
  }
  // rhoqc = (dens qc) 1000 (read by the effective radius)
  b_dens = fma(b_rhoqc * 1000.0, qc, b_dens);
  b_qc = fma(b_rhoqc * 1000.0, dens, b_qc);
  // Pracs = (K_racs Rdens) dvrs (2 MOMs_0bs RLMDr_3 + 2 MOMs_1bs RLMDr_2 + MOMs_2bs RLMDr)
  double b_dvrs = 0.0;
  {
    const double b_s = bPracs * racs_kd;
    const double b_kd = bPracs * racs_s;
    b_dvrs = fma(b_kd, racs_k, b_dvrs);
    b_Rdens = fma(b_kd * dvrs, C.K_racs, b_Rdens);
    b_mom[2] = fma(b_s * RLMDr_3, 2.0, b_mom[2]);
    b_RLMDr_3 = fma(b_s, racs_t1, b_RLMDr_3);
    b_mom[3] = fma(b_s * RLMDr_2, 2.0, b_mom[3]);
    b_RLMDr_2 = fma(b_s, racs_t2, b_RLMDr_2);
    b_mom[4] = fma(b_s, RLMDr, b_mom[4]);
    b_RLMDr = fma(b_s, MOMs_2bs, b_RLMDr);
  }
  // Pgacr = (K_gacr Rdens) |Vtg - Vtr| (K_g13 RLMDr_1br RLMDg_3 + K_g22 RLMDr_2br RLMDg_2 + GAM_3br RLMDr_3br RLMDg)
  {
    const double b_s = bPgacr * gacr_kd;
    const double b_kd = bPgacr * gacr_s;
    const double b_dv = b_kd * gacr_k;
    b_Rdens = fma(b_kd * dvgr, C.K_gacr, b_Rdens);
    const double sgn = dvgr_d < 0.0 ? -1.0 : 1.0;
    b_Vtg = fma(b_dv, sgn, b_Vtg);
    b_Vtr = fma(-b_dv, sgn, b_Vtr);
    b_RLMDr_1br = fma(b_s * RLMDg_3, C.K_g13, b_RLMDr_1br);
    b_RLMDg_3 = fma(b_s, gacr_t1, b_RLMDg_3);
    b_RLMDr_2br = fma(b_s * RLMDg_2, C.K_g22, b_RLMDr_2br);
    b_RLMDg_2 = fma(b_s, gacr_t2, b_RLMDg_2);
    b_RLMDr_3br = fma(b_s * RLMDg, C.GAM_3br, b_RLMDr_3br);
    b_RLMDg = fma(b_s, gacr_t3, b_RLMDg);
  }
  // Psacr = (K_sacr Rdens) dvrs (GAM_1br RLMDr_1br MOMs_2 + K_2gam2br RLMDr_2br MOMs_1 + GAM_3br RLMDr_3br MOMs_0)
  {
    const double b_s = bPsacr * sacr_kd;
    const double b_kd = bPsacr * sacr_s;
    b_dvrs = fma(b_kd, sacr_k, b_dvrs);
    b_Rdens = fma(b_kd * dvrs, C.K_sacr, b_Rdens);
    b_RLMDr_1br = fma(b_s * MOMs_2, C.GAM_1br, b_RLMDr_1br);
    b_MOMs_2 = fma(b_s, sacr_t1, b_MOMs_2);
    b_RLMDr_2br = fma(b_s * MOMs_1, C.K_2gam2br, b_RLMDr_2br);
    b_mom[1] = fma(b_s, sacr_t2, b_mom[1]);
    b_RLMDr_3br = fma(b_s * MOMs_0, C.GAM_3br, b_RLMDr_3br);
    b_mom[0] = fma(b_s, sacr_t3, b_mom[0]);
  }
  // dvrs = |Vtr - Vts|
  {
    const double sgn = dvrs_d < 0.0 ? -1.0 : 1.0;
    b_Vtr = fma(b_dvrs, sgn, b_Vtr);
    b_Vts = fma(-b_dvrs, sgn, b_Vts);
  }
  // Piacr = ((qi K_iacr) RLMDr_6dr) fr
  b_rho_fact = fma(bPiacr, iacr_b, b_rho_fact);
  {
    const double b_b = bPiacr * fr;
    b_RLMDr_6dr = fma(b_b, iacr_a, b_RLMDr_6dr);
    const double b_a = b_b * RLMDr_6dr;
    b_qi = fma(b_a, C.K_iacr, b_qi);
    b_K_iacr = fma(b_a, qi, b_K_iacr);
  }
  // Psaci = (((qi K_saci) Esi_mod) MOMs_2ds) fr
  b_rho_fact = fma(bPsaci, saci_c, b_rho_fact);
  {
    const double b_c = bPsaci * fr;
    b_mom[5] = fma(b_c, saci_b, b_mom[5]);
    const double b_b = b_c * MOMs_2ds;
    b_Esi_mod = fma(b_b, saci_a, b_Esi_mod);
    const double b_a = b_b * Esi_mod;
    b_qi = fma(b_a, C.K_saci, b_qi);
    b_K_saci = fma(b_a, qi, b_K_saci);
  }
  // Praci = ((qi K_raci) RLMDr_3dr) fr
  b_rho_fact = fma(bPraci, raci_b, b_rho_fact);
  {
    const double b_b = bPraci * fr;
    b_RLMDr_3dr = fma(b_b, raci_a, b_RLMDr_3dr);
    const double b_a = b_b * RLMDr_3dr;
    b_qi = fma(b_a, C.K_raci, b_qi);
    b_K_raci = fma(b_a, qi, b_K_raci);
  }
  // Pgacw = ((qc K_gacw) RLMDg_3dg) fr
  b_rho_fact = fma(bPgacw, gacw_b, b_rho_fact);
  {
    const double b_b = bPgacw * fr;
    b_RLMDg_3dg = fma(b_b, gacw_a, b_RLMDg_3dg);
    const double b_a = b_b * RLMDg_3dg;
    b_qc = fma(b_a, C.K_gacw, b_qc);
    b_K_gacw = fma(b_a, qc, b_K_gacw);
  }
  // Psacw = ((qc K_sacw) MOMs_2ds) fr
  b_rho_fact = fma(bPsacw, sacw_b, b_rho_fact);
  {
    const double b_b = bPsacw * fr;
    b_mom[5] = fma(b_b, sacw_a, b_mom[5]);
    const double b_a = b_b * MOMs_2ds;
    b_qc = fma(b_a, C.K_sacw, b_qc);
    b_K_sacw = fma(b_a, qc, b_K_sacw);
  }
  // Pracw = 67 pow(qc qr, 1.15)
  if (prw_on) {
    const double b_pow = bPracw0 * 67.0;
    if (qcqr > 0.0) {
      const double b_qcqr = b_pow * 1.15 * prw_pow / qcqr;
      b_qc = fma(b_qcqr, qr, b_qc);
      b_qr = fma(b_qcqr, qc, b_qr);
    }
  }
  // Esi_mod = min(Esi, Esi eg), betai = min(beta, beta eg), eg = exp(gamma_sacr temc)
  if (cold_branch) {
    double b_eg = 0.0;
    if (esi_exp) b_eg += b_Esi_mod * C.Esi;
    if (bet_exp) {
      b_eg = fma(b_betai, C.beta_saut, b_eg);
      b_beta = fma(b_betai, eg, b_beta);
    } else {
      b_beta += b_betai;
    }
    b_temc = fma(b_eg * eg, C.gamma_sacr, b_temc);
  } else {
    b_beta += b_betai;
  }
  // Pigen = max(min(Qi0 - qi, qv - qsati), 0) rdt
  {
    const double b_max = bPigen * rdt;
    double b_min = 0.0, dummy = 0.0;
    bmax(pgmin, Z, b_max, b_min, dummy);
    double b_p1 = 0.0, b_p2 = 0.0;
    bmin(pg1, pg2, b_min, b_p1, b_p2);
    b_qi -= b_p1;
    b_qv += b_p2;
    b_qsati -= b_p2;
    // Qi0 = (ice_nuc exp(1.33 (ln1000 + max(-0.1 temc, 0)))) Rdens
    b_Rdens = fma(b_p1, qi0a, b_Rdens);
    const double b_qi0a = b_p1 * Rdens;
    b_icenuc = fma(b_qi0a, nexp, b_icenuc);
    const double b_nex = b_qi0a * C.ice_nuc * nexp;
    double b_nm01 = 0.0, dummy2 = 0.0;
    bmax(nm01, Z, b_nex * 1.33, b_nm01, dummy2);
    b_temc = fma(b_nm01, -0.1, b_temc);
  }
  // terminal velocities: Vtr = (K_vtr rho_fact) RLMDr_dr etc.
  {
    b_RLMDr_dr = fma(b_Vtr, vtr_a, b_RLMDr_dr);
    const double b_a = b_Vtr * RLMDr_dr;
    b_K_vtr = fma(b_a, rho_fact, b_K_vtr);
    b_rho_fact = fma(b_a, C.K_vtr, b_rho_fact);
    b_RMOMs_Vt = fma(b_Vts, vts_a, b_RMOMs_Vt);
    const double b_s = b_Vts * RMOMs_Vt;
    b_K_vts = fma(b_s, rho_fact, b_K_vts);
    b_rho_fact = fma(b_s, C.K_vts, b_rho_fact);
    b_RLMDg_dg = fma(b_Vtg, vtg_a, b_RLMDg_dg);
    const double b_g = b_Vtg * RLMDg_dg;
    b_K_vtg = fma(b_g, rho_fact, b_K_vtg);
    b_rho_fact = fma(b_g, C.K_vtg, b_rho_fact);
  }
  // graupel slope parameter
  if (graupel) {
    b_RLMDg_3 = fma(b_RLMDg_5dg * RLMDg_dg, RLMDg_2, b_RLMDg_3);
    b_RLMDg_2 = fma(b_RLMDg_5dg * RLMDg_dg, RLMDg_3, b_RLMDg_2);
    b_RLMDg_dg = fma(b_RLMDg_5dg, g32, b_RLMDg_dg);
    b_RLMDg_3 = fma(b_RLMDg_3dg, RLMDg_dg, b_RLMDg_3);
    b_RLMDg_dg = fma(b_RLMDg_3dg, RLMDg_3, b_RLMDg_dg);
    b_RLMDg_2 = fma(b_RLMDg_3, RLMDg, b_RLMDg_2);
    b_RLMDg = fma(b_RLMDg_3, RLMDg_2, b_RLMDg);
    b_RLMDg = fma(b_RLMDg_2 * 2.0, RLMDg, b_RLMDg);
    b_RLMDg = fma(b_RLMDg_dg, bsqrt(RLMDg_dg), b_RLMDg);
    const double b_s1 = b_RLMDg * bsqrt(RLMDg);
    const double b_b = b_s1 * bsqrt(g_s1);
    const double b_a = b_b * C.K_rlmdg;
    b_dens = fma(b_a, qg, b_dens);
    b_qg = fma(b_a, dens, b_qg);
  }
  // snow moments: Vts's RMOMs_Vt = mom5 / mom2; mom_i = exp(logX lb_i + la_i(tems)); MOMs_2 = Xs2
  double b_Xs2 = b_MOMs_2;
  if (snow) {
    const double rm2 = 1.0 / mom[2];
    b_mom[5] = fma(b_RMOMs_Vt, rm2, b_mom[5]);
    b_mom[2] = fma(-(b_RMOMs_Vt * RMOMs_Vt), rm2, b_mom[2]);
    double b_logX = 0.0, b_tems = 0.0;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const double b_arg = b_mom[i] * mom[i];
      b_logX = fma(b_arg, mlb[i], b_logX);
      const double* a = C.roh_a + 4 * i;
      const double* b = C.roh_b + 4 * i;
      // d la / d tems and d lb / d tems of the cubics
      const double dla = __fma_rn(__fma_rn(3.0 * a[3], tems, 2.0 * a[2]), tems, a[1]);
      const double dlb = __fma_rn(__fma_rn(3.0 * b[3], tems, 2.0 * b[2]), tems, b[1]);
      b_tems = fma(b_arg, (dla + logX * dlb), b_tems);
    }
    b_Xs2 += b_logX / Xs2;
    if (tems_sel) b_temc += b_tems;
  }
  {
    const double b_xsa = b_Xs2 * C.rAs;
    b_dens = fma(b_xsa, qs, b_dens);
    b_qs = fma(b_xsa, dens, b_qs);
  }
  // rain slope parameter
  if (rain) {
    b_RLMDr_3br = fma(b_RLMDr_6dr, RLMDr_dr, b_RLMDr_3br);
    b_RLMDr_dr = fma(b_RLMDr_6dr, RLMDr_3br, b_RLMDr_dr);
    b_RLMDr_2br = fma(b_RLMDr_5dr, RLMDr_dr, b_RLMDr_2br);
    b_RLMDr_dr = fma(b_RLMDr_5dr, RLMDr_2br, b_RLMDr_dr);
    b_RLMDr_3 = fma(b_RLMDr_3dr, RLMDr_dr, b_RLMDr_3);
    b_RLMDr_dr = fma(b_RLMDr_3dr, RLMDr_3, b_RLMDr_dr);
    b_RLMDr_3br = fma(b_RLMDr_7, RLMDr, b_RLMDr_3br);
    b_RLMDr = fma(b_RLMDr_7, RLMDr_3br, b_RLMDr);
    b_RLMDr_3 = fma(b_RLMDr_3br * 2.0, RLMDr_3, b_RLMDr_3);
    b_RLMDr_1br = fma(b_RLMDr_2br, RLMDr, b_RLMDr_1br);
    b_RLMDr = fma(b_RLMDr_2br, RLMDr_1br, b_RLMDr);
    b_RLMDr_2 = fma(b_RLMDr_1br * 2.0, RLMDr_2, b_RLMDr_2);
    b_RLMDr_2 = fma(b_RLMDr_3, RLMDr, b_RLMDr_2);
    b_RLMDr = fma(b_RLMDr_3, RLMDr_2, b_RLMDr);
    b_RLMDr = fma(b_RLMDr_2 * 2.0, RLMDr, b_RLMDr);
    b_RLMDr = fma(b_RLMDr_dr, bsqrt(RLMDr_dr), b_RLMDr);
    const double b_s1 = b_RLMDr * bsqrt(RLMDr);
    const double b_b = b_s1 * bsqrt(r_s1);
    const double b_a = b_b * C.K_rlmdr;
    b_dens = fma(b_a, qr, b_dens);
    b_qr = fma(b_a, dens, b_qr);
  }
  // dq/dt = q / dt
  {
    const double rdt = 1.0 / dt;
    b_qv = fma(b_dqv, rdt, b_qv);
    b_qc = fma(b_dqc, rdt, b_qc);
    b_qr = fma(b_dqr, rdt, b_qr);
    b_qi = fma(b_dqi, rdt, b_qi);
    b_qs = fma(b_dqs, rdt, b_qs);
    b_qg = fma(b_dqg, rdt, b_qg);
  }
  // temc = temp - TEM00; rho_fact = sqrt(DENS00 Rdens); Rdens = 1 / dens
  b_temp += b_temc;
  b_Rdens = fma(b_rho_fact * bsqrt(rho_fact), DENS00, b_Rdens);
  b_dens = fma(-(b_Rdens * Rdens), Rdens, b_dens);
  // Sliq = qv / max(qsatl, EPS), Sice = qv / max(qsati, EPS)
  {
    const double rsld = 1.0 / sld;
    b_qv = fma(b_Sliq, rsld, b_qv);
    const double b_sld = -b_Sliq * Sliq * rsld;
    double dummy = 0.0;
    bmax(qsatl, EPS, b_sld, b_qsatl, dummy);
    const double rsid = 1.0 / sid;
    b_qv = fma(b_Sice, rsid, b_qv);
    const double b_sid = -b_Sice * Sice * rsid;
    bmax(qsati, EPS, b_sid, b_qsati, dummy);
  }
  // q* = max(qn, 0)
  double b_qn[6] = {0, 0, 0, 0, 0, 0};
  const double bq[6] = {b_qv, b_qc, b_qr, b_qi, b_qs, b_qg};
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    double dummy = 0.0;
    bmax(qn[n], Z, bq[n], b_qn[n], dummy);
  }
  // psat / qsat: qsat = psat (1 / ((dens RVAP) temp)), psat = PSAT0 exp(LovR (RTEM00 - rtem))
  {
    const double b_rdrt = b_qsatl * psatl + b_qsati * psati;
    const double b_psatl = b_qsatl * rdrt, b_psati = b_qsati * rdrt;
    const double b_drt = -b_rdrt * rdrt * rdrt;
    b_dens = fma(b_drt * temp, RVAP, b_dens);
    b_temp = fma(b_drt, drv, b_temp);
    b_rtem -= b_psatl * PSAT0 * el * C.LovR_liq + b_psati * PSAT0 * ei * C.LovR_ice;
    // rtem = 1 / max(temp, TEM_MIN)
    const double b_tmx = -b_rtem * rtem * rtem;
    double dummy = 0.0;
    bmax(temp, TEM_MIN, b_tmx, b_temp, dummy);
  }
  // pre = (dens (qd RDRY + qn0 RVAP)) temp
  {
    b_temp = fma(b_pre, dp, b_temp);
    const double b_dp = b_pre * temp;
    b_dens = fma(b_dp, pq, b_dens);
    const double b_pq = b_dp * dens;
    double b_qd = b_pq * RDRY;
    b_qn[0] = fma(b_pq, RVAP, b_qn[0]);
    // rhoge0 = (temp rhog) cv
    const double b_trh = b_rhoge0 * cv;
    const double b_cv = b_rhoge0 * trh;
    b_temp = fma(b_trh, rhog, b_temp);
    b_rhog = fma(b_trh, temp, b_rhog);
    b_qd = fma(b_cv, CVDRY, b_qd);
#pragma unroll
    for (int n = 1; n <= 5; ++n) b_qn[n] += b_cv * CVDRY - b_qd;
  }
  // qn[n] = rq[n] / rhog (n >= 1); dens = rhog / gsgam2
  {
#pragma unroll
    for (int n = 1; n <= 5; ++n) {
      b_rq[n] = fma(b_qn[n], rrhog, b_rq[n]);
      b_rhog = fma(-(b_qn[n] * qn[n]), rrhog, b_rhog);
    }
    const double rgs = 1.0 / in.gsgam2;
    b_rhog = fma(b_dens, rgs, b_rhog);
    ib.gsgam2 = fma(-b_dens * dens, rgs, ib.gsgam2);
  }
  // rhog = in.rhog (1 - d2); negative filter
  {
    ib.rhog = fma(b_rhog, omd, ib.rhog);
    const double b_d2 = -b_rhog * in.rhog;
    // d2 = rq0a - clip(rq0a): d d2 / d rq0a = clip ? 1 : 0; rq[0] = clip(rq0a)
    const double b_rq0a = (clip[0] ? b_d2 : 0.0) + (clip[0] ? 0.0 : b_rq[0]);
    // rq0a = rq_in0 + diffq; diffq = sum_{clipped} rq_in[n]
    ib.rhogq[0] += b_rq0a;
#pragma unroll
    for (int n = 2; n <= 5; ++n) ib.rhogq[n] += (clip[n] ? b_rq0a : 0.0) + (clip[n] ? 0.0 : b_rq[n]);
    ib.rhogq[1] += b_rq[1];
  }
  ib.tem += b_temp;
  ib.q0 += b_qn[0];
  // parameters
  pb[0] += b_beta;
  pb[1] += b_qicrt;
  pb[2] += (b_K_vtr * C.K_vtr + b_K_raci * C.K_raci + b_K_iacr * C.K_iacr) * (1.0 / C.Cr) + b_Cr;
  pb[3] += (b_K_vts * C.K_vts + b_K_sacw * C.K_sacw + b_K_saci * C.K_saci + b_K_vents2 * 0.5 * C.K_vents2) *
           (1.0 / C.Cs);
  pb[4] += (b_K_vtg * C.K_vtg + b_K_gacw * C.K_gacw) * (1.0 / C.Cg) + b_Cg;
  pb[5] += b_icenuc;
  pb[6] += b_K_aut * C.K_aut / C.kk_aut;
}

#undef NSW6_CK

}  // namespace nsw6
