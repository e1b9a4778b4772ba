// Per-cell NSW6 physics (device), FP64.
//
// One call evaluates, for one interior cell, what the reference computes in
// several whole-field passes: negative_filter (mod_mp_nsw6.cpp:1750-1832),
// saturation vapour pressure and mixing ratio (mod_satadjust.cpp:80-160,
// mod_mp_nsw6.cpp:686-690), the TagBigLoop process rates
// (mod_mp_nsw6.cpp:760-1594) and the cell updates TagUpdateRHOGQ / RHOGE /
// MassConc / TEM (mod_mp_nsw6.cpp:692-744).
//
// The FP64 pipe is the bottleneck on GB300, so the arithmetic is organised to
// issue as few FP64 instructions as possible while staying within a few units
// in the last place of the reference:
//
//  * terms the configuration fixed by mp_nsw6_init multiplies by an exact
//    zero are not evaluated: sw_expice = 1 makes the Bergeron terms Psfw, Psfi
//    (and Bergeron_param) vanish (sw_bergeron = 0, :932-934); sw_kk2000 = 1
//    drops the Berry and "orig" rates (:1094-1099, :1158-1160); sw_roh2014 = 1
//    replaces the classic snow moments (:982-992 are dead); Egi = Egs = 0 and
//    beta_gaut = 0 make Pgaci, Pgacs and Pgaut vanish; the ice fall speed Vti
//    is not used because QI does not sediment ("3WATER");
//  * products of constants are folded on the host, divisions by a shared
//    denominator use one reciprocal, and integer powers are products;
//  * exp / log / pow come from a math policy: FastMath (table-driven, see
//    nsw6_fastmath.cuh) in production, LibMath (CUDA's libm) for checks.
//
// Removing the dead terms is exact except for the sign of zero results.
#pragma once

#include "nsw6_common.cuh"
#include "nsw6_fastmath.cuh"

namespace nsw6 {

// a / b rounded to nearest, given rb = 1 / b rounded to nearest: one product
// and Markstein's correction step (r = a - q b is exact in an FMA, and q + r rb
// rounds to the correctly rounded quotient).  Three FP64 instructions where a
// division costs several times more; used where the reference divides by a
// value the cell reuses, so that near-total consumption of a species leaves
// the same residue as in the reference.
__device__ __forceinline__ double div_rn(double a, double b, double rb) {
  const double q = a * rb;
  const double r = __fma_rn(-q, b, a);
  return __fma_rn(r, rb, q);
}

struct CellIn {
  double rhog, tem, gsgam2, q0;
  double rhogq[6];
};

struct CellOut {
  double rhog, rhoge, tem;
  double rhogq[6];
  double q[6];
  double Vtr, Vts, Vtg;
  double rceff, rceff_cld, rctop, tctop;
};

template <class M>
__device__ __forceinline__ void nsw6_cell(const Consts& C, const M& mth, double dt, double rdt, const CellIn& in,
                                          CellOut& o) {
  // ---- negative_filter, mod_mp_nsw6.cpp:1770-1831
  double rq[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] = in.rhogq[n];
  double diffq = 0.0;
#pragma unroll
  for (int n = 2; n <= 5; ++n) {
    diffq += rq[n];
    rq[n] = dmax(rq[n], 0.0);
  }
#pragma unroll
  for (int n = 2; n <= 5; ++n) diffq -= rq[n];
  rq[I_QV] += diffq;
  diffq = rq[I_QV];
  rq[I_QV] = dmax(rq[I_QV], 0.0);
  diffq -= rq[I_QV];
  const double rhog = in.rhog * (1.0 - diffq);
  const double rrhog = 1.0 / rhog;
  const double dens = rhog / in.gsgam2;
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
  double rhoge = temp * rhog * cv;
  const double pre = dens * (qd * RDRY + qn[0] * RVAP) * temp;

  // ---- psat / qsat (CPovR = 0 under EIN_TYPE "SIMPLE": the power term is 1)
  const double rtem = 1.0 / dmax(temp, TEM_MIN);
  const double psatl = PSAT0 * mth.exp(C.LovR_liq * (C.RTEM00 - rtem));
  const double psati = PSAT0 * mth.exp(C.LovR_ice * (C.RTEM00 - rtem));
  const double rdrt = 1.0 / (dens * RVAP * temp);
  const double qsatl = psatl * rdrt;
  const double qsati = psati * rdrt;

  // ---- TagBigLoop, mod_mp_nsw6.cpp:902-1594
  const double qv = dmax(qn[0], 0.0), qc = dmax(qn[1], 0.0), qr = dmax(qn[2], 0.0);
  const double qi = dmax(qn[3], 0.0), qs = dmax(qn[4], 0.0), qg = dmax(qn[5], 0.0);
  const double Sliq = qv / dmax(qsatl, EPS);
  const double Sice = qv / dmax(qsati, EPS);
  const double Rdens = 1.0 / dens;
  const double rho_fact = sqrt(DENS00 * Rdens);
  const double temc = temp - TEM00;
  const bool warm = !(temc < 0.0);  // iceflg = 0.5 - copysign(0.5, temc) == 0
  const double iceflg = warm ? 0.0 : 1.0;
  const double delta1 = (qr >= 1.0E-4) ? 1.0 : 0.0;
  const double delta2 = (1.0E-4 >= qr && 1.0E-4 >= qs) ? 1.0 : 0.0;
  const double spsati = (Sice >= 1.0) ? 1.0 : 0.0;
  const double dqv_dt = div_rn(qv, dt, rdt), dqc_dt = div_rn(qc, dt, rdt), dqr_dt = div_rn(qr, dt, rdt);
  const double dqi_dt = div_rn(qi, dt, rdt), dqs_dt = div_rn(qs, dt, rdt), dqg_dt = div_rn(qg, dt, rdt);

  // rain slope parameter, :953-967
  const double RLMDr = (qr >= 1.0E-12) ? sqrt(sqrt(dens * qr * C.K_rlmdr)) : 0.0;
  const double RLMDr_dr = sqrt(RLMDr);
  const double RLMDr_2 = RLMDr * RLMDr;
  const double RLMDr_3 = RLMDr_2 * RLMDr;
  const double RLMDr_1br = RLMDr_2 * RLMDr_2;
  const double RLMDr_2br = RLMDr_1br * RLMDr;
  const double RLMDr_3br = RLMDr_3 * RLMDr_3;
  const double RLMDr_7 = RLMDr_3br * RLMDr;
  const double RLMDr_3dr = RLMDr_3 * RLMDr_dr;
  const double RLMDr_5dr = RLMDr_2br * RLMDr_dr;
  const double RLMDr_6dr = RLMDr_3br * RLMDr_dr;

  // Roh and Satoh (2014) snow moments, :994-1057.  Each moment is
  // 10^loga * Xs2^b = exp(ln10 * loga + log(Xs2) * b), with loga and b
  // polynomials in tems whose coefficients per moment are folded on the host.
  const double Xs2 = dens * qs * C.rAs;
  const bool snow = (Xs2 >= 1.0E-12);
  const double tems = dmin(-0.1, temc);
  const double logX = snow ? mth.log(Xs2) : 0.0;
  double mom[7];  // MOMs_0, MOMs_1, MOMs_0bs, MOMs_1bs, MOMs_2bs, MOMs_2ds (= nm 2.25), MOMs_5ds_h
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    const double* a = C.roh_a + 4 * i;
    const double* b = C.roh_b + 4 * i;
    const double la = __fma_rn(__fma_rn(__fma_rn(a[3], tems, a[2]), tems, a[1]), tems, a[0]);
    const double lb = __fma_rn(__fma_rn(__fma_rn(b[3], tems, b[2]), tems, b[1]), tems, b[0]);
    mom[i] = snow ? mth.exp(__fma_rn(logX, lb, la)) : 0.0;
  }
  const double MOMs_0 = mom[0], MOMs_1 = mom[1], MOMs_2 = Xs2;
  const double MOMs_0bs = mom[2], MOMs_1bs = mom[3], MOMs_2bs = mom[4], MOMs_2ds = mom[5];
  const double MOMs_5ds_h = mom[6];
  const double RMOMs_Vt = snow ? mom[5] / MOMs_0bs : 0.0;

  // graupel slope parameter, :1059-1066
  const double RLMDg = (qg >= 1.0E-12) ? sqrt(sqrt(dens * qg * C.K_rlmdg)) : 0.0;
  const double RLMDg_dg = sqrt(RLMDg);
  const double RLMDg_2 = RLMDg * RLMDg;
  const double RLMDg_3 = RLMDg_2 * RLMDg;
  const double RLMDg_3dg = RLMDg_3 * RLMDg_dg;
  const double RLMDg_5dg = RLMDg_3 * RLMDg_2 * RLMDg_dg;

  // terminal velocity, :1072-1078
  const double Vtr = C.K_vtr * rho_fact * RLMDr_dr;
  const double Vts = C.K_vts * rho_fact * RMOMs_Vt;
  const double Vtg = C.K_vtg * rho_fact * RLMDg_dg;

  // nucleation, :1080-1085: Ni0 = max(exp(-0.1 temc), 1) * 1000 and
  // Qi0 = ice_nuc * Ni0^1.33 / dens, with log(Ni0) = ln 1000 + max(-0.1 temc, 0)
  const double Qi0 = C.ice_nuc * mth.exp(1.33 * (C.ln1000 + dmax(-0.1 * temc, 0.0))) * Rdens;
  double Pigen = dmax(dmin(Qi0 - qi, qv - qsati), 0.0) * rdt;

  // accretion, :1087-1145
  const double Esi_mod = dmin(C.Esi, C.Esi * mth.exp(C.gamma_sacr * temc));
  const double qcqr = qc * qr;
  double Pracw = (qcqr >= 1.0E-12) ? 67.0 * mth.pow(qcqr, 1.15) : 0.0;
  const double fr = rho_fact;
  double Psacw = qc * C.K_sacw * MOMs_2ds * fr;
  double Pgacw = qc * C.K_gacw * RLMDg_3dg * fr;
  double Praci = qi * C.K_raci * RLMDr_3dr * fr;
  double Psaci = qi * C.K_saci * Esi_mod * MOMs_2ds * fr;
  double Piacr = qi * C.K_iacr * RLMDr_6dr * fr;
  const double dvrs = fabs(Vtr - Vts);
  double Psacr = C.K_sacr * Rdens * dvrs *
                 (C.GAM_1br * RLMDr_1br * MOMs_2 + C.K_2gam2br * RLMDr_2br * MOMs_1 + C.GAM_3br * RLMDr_3br * MOMs_0);
  double Pgacr = C.K_gacr * Rdens * fabs(Vtg - Vtr) *
                 (C.K_g13 * RLMDr_1br * RLMDg_3 + C.K_g22 * RLMDr_2br * RLMDg_2 + C.GAM_3br * RLMDr_3br * RLMDg);
  double Pracs = C.K_racs * Rdens * dvrs * (2.0 * MOMs_0bs * RLMDr_3 + 2.0 * MOMs_1bs * RLMDr_2 + MOMs_2bs * RLMDr);

  // autoconversion, :1147-1172 (KK2000; only the second Praut_kk assignment is live)
  const double rhoqc = dens * qc * 1000.0;
  double Praut = C.K_aut * mth.pow(qc, 2.47);
  const double betai = dmin(C.beta_saut, C.beta_saut * mth.exp(C.gamma_saut * temc));
  double Psaut = dmax(betai * (qi - C.qicrt_saut), 0.0);

  // evaporation, sublimation, melting and freezing, :1174-1247
  const double Ka = (2.428E-2 + 7.47E-5 * temc);
  const double KdD = (2.222E-5 + 1.37E-7 * temc) * PSTD / pre * dens;   // Kd * dens
  const double rNu = dens / (1.718E-5 + 5.28E-8 * temc);                // 1 / Nu
  const double rKaT = 1.0 / (Ka * temp);
  const double xl = KdD * qsatl, xi = KdD * qsati;
  const double Glv = xl / (LHV0 * rKaT * (C.LovR_liq * rtem - 1.0) * xl + 1.0);
  const double Giv = xi / (LHS0 * rKaT * (C.LovR_ice * rtem - 1.0) * xi + 1.0);
  const double Gil = Ka * temc * C.rLHF0;
  const double ventr = C.K_ventr1 * RLMDr_2 + C.K_ventr2 * sqrt(C.Cr * fr * rNu * RLMDr_5dr);
  double Prevp = C.K_revp * Rdens * (1.0 - dmin(Sliq, 1.0)) * Glv * ventr;
  const double rhoqi = dmax(dens * qi, EPS);
  const double XNi = dmin(dmax(5.38E+7 * mth.pow(rhoqi, 0.75), 1.0E+3), 1.0E+6);
  const double XMi = rhoqi / XNi;
  const double Di = dmin(C.Di_a * sqrt(XMi), C.Di_max);
  double tmp = 4.0 * Di * XNi * Rdens * (Sice - 1.0) * Giv;
  double Pidep = spsati * tmp;
  double Pisub = (1.0 - spsati) * (-tmp);
  const bool below40 = (temc + 40.0 < 0.0);
  double Pihom = below40 ? dqc_dt : 0.0;
  const double efrz = mth.exp(-C.A_frz * temc) - 1.0;
  double Pihtr = (!below40 && !warm) ? dens * (qc * qc) * C.K_ihtr * efrz : 0.0;
  double Pimlt = warm ? dqi_dt : 0.0;
  const double vents = 0.65 * MOMs_1 + C.K_vents2 * sqrt(fr * rNu) * MOMs_5ds_h;
  tmp = C.K_2pi * Rdens * (Sice - 1.0) * Giv * vents;
  double Psdep = spsati * tmp;
  double Pssub = (1.0 - spsati) * (-tmp);
  double Psmlt = dmax(C.K_2pi * Rdens * Gil * vents + C.K_clf * temc * (Psacw + Psacr), 0.0);
  const double ventg = C.K_ventg1 * RLMDg_2 + C.K_ventg2 * sqrt(C.Cg * fr * rNu * RLMDg_5dg);
  tmp = C.K_gdep * Rdens * (Sice - 1.0) * Giv * ventg;
  double Pgdep = spsati * tmp;
  double Pgsub = (1.0 - spsati) * (-tmp);
  double Pgmlt = dmax(C.K_gdep * Rdens * Gil * ventg + C.K_clf * temc * (Pgacw + Pgacr), 0.0);
  double Pgfrz = C.K_gfrz * Rdens * efrz * RLMDr_7;

  // limiters, :1249-1296 (iceflg selects; sw_expice = 1; Psfw = Psfi = Pgaut = Pgaci = Pgacs = 0)
  Pigen = dmin(Pigen, dqv_dt) * iceflg;
  Pidep = dmin(Pidep, dqv_dt) * iceflg;
  Psdep = dmin(Psdep, dqv_dt) * iceflg;
  Pgdep = dmin(Pgdep, dqv_dt) * iceflg;
  Pracw = Pracw + Psacw * (1.0 - iceflg) + Pgacw * (1.0 - iceflg);
  Praut = dmin(Praut, dqc_dt);
  Pracw = dmin(Pracw, dqc_dt);
  Pihom = dmin(Pihom, dqc_dt) * iceflg;
  Pihtr = dmin(Pihtr, dqc_dt) * iceflg;
  Psacw = dmin(Psacw, dqc_dt) * iceflg;
  Pgacw = dmin(Pgacw, dqc_dt) * iceflg;
  Prevp = dmin(Prevp, dqr_dt);
  Piacr = dmin(Piacr, dqr_dt) * iceflg;
  Psacr = dmin(Psacr, dqr_dt) * iceflg;
  Pgacr = dmin(Pgacr, dqr_dt) * iceflg;
  Pgfrz = dmin(Pgfrz, dqr_dt) * iceflg;
  Pisub = dmin(Pisub, dqi_dt) * iceflg;
  Pimlt = dmin(Pimlt, dqi_dt) * (1.0 - iceflg);
  Psaut = dmin(Psaut, dqi_dt) * iceflg;
  Praci = dmin(Praci, dqi_dt) * iceflg;
  Psaci = dmin(Psaci, dqi_dt) * iceflg;
  Pssub = dmin(Pssub, dqs_dt) * iceflg;
  Psmlt = dmin(Psmlt, dqs_dt) * (1.0 - iceflg);
  Pracs = dmin(Pracs, dqs_dt) * iceflg;
  Pgsub = dmin(Pgsub, dqg_dt) * iceflg;
  Pgmlt = dmin(Pgmlt, dqg_dt) * (1.0 - iceflg);
  double Piacr_s = (1.0 - delta1) * Piacr;
  double Piacr_g = delta1 * Piacr;
  double Praci_s = (1.0 - delta1) * Praci;
  double Praci_g = delta1 * Praci;
  double Psacr_s = delta2 * Psacr;
  double Psacr_g = (1.0 - delta2) * Psacr;
  Pracs = (1.0 - delta2) * Pracs;

  // loss limiters, :1298-1477: fac = 1 when production >= loss - EPS,
  // else min(-dq/dt / net, 1) (the reference's (net - fac_sw) is net there)
  auto limiter = [&](double net, double dq) {
    return (net + EPS >= 0.0) ? 1.0 : dmin(-dq / net, 1.0);
  };
  double fac;
  fac = limiter(+Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw, dqc_dt);  // [QC]
  Pimlt *= fac; Praut *= fac; Pracw *= fac; Pihom *= fac; Pihtr *= fac; Psacw *= fac; Pgacw *= fac;
  fac = limiter(+Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g, dqi_dt);  // [QI]
  Pigen *= fac; Pidep *= fac; Pihom *= fac; Pihtr *= fac; Pisub *= fac; Pimlt *= fac; Psaut *= fac;
  Praci_s *= fac; Psaci *= fac; Praci_g *= fac;
  fac = limiter(+Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz,
                dqr_dt);  // [QR]
  Praut *= fac; Pracw *= fac; Psmlt *= fac; Pgmlt *= fac; Prevp *= fac; Piacr_s *= fac; Psacr_s *= fac;
  Piacr_g *= fac; Psacr_g *= fac; Pgacr *= fac; Pgfrz *= fac;
  fac = limiter(+Prevp + Pisub + Pssub + Pgsub - Pigen - Pidep - Psdep - Pgdep, dqv_dt);  // [QV]
  Prevp *= fac; Pisub *= fac; Pssub *= fac; Pgsub *= fac; Pigen *= fac; Pidep *= fac; Psdep *= fac; Pgdep *= fac;
  fac = limiter(+Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs, dqs_dt);  // [QS]
  Psdep *= fac; Psacw *= fac; Piacr_s *= fac; Psacr_s *= fac; Psaut *= fac; Praci_s *= fac; Psaci *= fac;
  Pssub *= fac; Psmlt *= fac; Pracs *= fac;
  fac = limiter(+Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt, dqg_dt);  // [QG]
  Pgdep *= fac; Pgacw *= fac; Piacr_g *= fac; Psacr_g *= fac; Pgacr *= fac; Pgfrz *= fac; Praci_g *= fac;
  Pracs *= fac; Pgsub *= fac; Pgmlt *= fac;

  // tendencies, :1479-1559
  double qc_t = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw;
  double qr_t = +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz;
  double qi_t = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g;
  double qs_t = +Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs;
  double qg_t = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt;
  qc_t = dmax(qc_t, -dqc_dt);
  qr_t = dmax(qr_t, -dqr_dt);
  qi_t = dmax(qi_t, -dqi_dt);
  qs_t = dmax(qs_t, -dqs_dt);
  qg_t = dmax(qg_t, -dqg_dt);
  const double qv_t = -(qc_t + qr_t + qi_t + qs_t + qg_t);
  double drq[6];
  drq[0] = rhog * qv_t * dt;
  drq[1] = rhog * qc_t * dt;
  drq[2] = rhog * qr_t * dt;
  drq[3] = rhog * qi_t * dt;
  drq[4] = rhog * qs_t * dt;
  drq[5] = rhog * qg_t * dt;
  o.Vtr = Vtr;
  o.Vts = Vts;
  o.Vtg = Vtg;

  // effective radius and cloud top, :1566-1592
  {
    const double r2_min = 1.0E-10, q_min = 1.0E-5;
    const double rf_qc = mth.pow(C.coef_xf * (rhoqc * C.K_xf) + EPS, 0.33333333);
    const double r2_qc = C.K_r2c * (rf_qc * rf_qc);
    const double r2_qr = C.K_r2r * RLMDr_3;
    const double r3_qc = C.coef_xf * dens * qc;
    const double r3_qr = C.coef_xf * dens * qr;
    const double r2 = r2_qc + r2_qr;
    const bool big = (r2 >= r2_min);
    o.rceff = big ? (r3_qc + r3_qr) / r2 : 0.0;
    const bool top = !big && ((qc + qr) >= q_min);
    o.rctop = top ? o.rceff : UNDEF;
    o.tctop = top ? temp : UNDEF;
    o.rceff_cld = (r2_qc >= r2_min) ? r3_qc / r2_qc : 0.0;
  }

  // ---- TagUpdateRHOGQ / RHOGE / MassConc / TEM, mod_mp_nsw6.cpp:692-744
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] += drq[n];
  rhoge = rhoge - LHV0 * drq[I_QV] + LHF0 * drq[I_QI] + LHF0 * drq[I_QS] + LHF0 * drq[I_QG];
  o.q[0] = qn[0];
#pragma unroll
  for (int n = 1; n <= 5; ++n) o.q[n] = div_rn(rq[n], rhog, rrhog);
  double qd2 = 1.0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qd2 = qd2 - o.q[n];
  double cva = qd2 * CVDRY;
#pragma unroll
  for (int n = 1; n <= 5; ++n) cva = cva + o.q[n] * CVDRY;
  o.tem = rhoge / (rhog * cva);
  o.rhog = rhog;
  o.rhoge = rhoge;
#pragma unroll
  for (int n = 0; n < 6; ++n) o.rhogq[n] = rq[n];
}

// Half-level velocity wh(j) of vadv1d_prep (mod_vadv1d.cpp:270-282) for a column
// accessor wp(j).
template <class WP>
__device__ __forceinline__ double vadv_wh(const WP& wp, int j, int mkmin, int mkmax) {
  if (j >= mkmin + 1 && j <= mkmax) return 0.5 * (wp(j - 1) + wp(j));
  if (j == mkmin) return wp(mkmin);
  if (j == mkmin - 1) return wp(mkmin - 1);
  return wp(mkmax);  // j == mkmax + 1
}

// Departure distance zdis(k) of vadv1d_prep for k in [mkmin, mkmax]
// (mod_vadv1d.cpp:284-302):
//   zdis = dt w - dt^2/2 w (w+ - w-)/(dz- + dz) + dt^3/6 w (r^2 + w c),
//   r = (w+ - w-)/(dz- + dz),  c = 2 ((w+ - w)/dz - (w - w-)/dz-)/(dz- + dz),
// evaluated with the per-level reciprocals rdz = 1/dz and rdzs = 1/(dz- + dz)
// instead of divisions.  zdis only decides which layer the departure point
// lies in (an ulp-level change matters only within an ulp of an interface)
// and scales the flux of the departure layer.
template <class WP>
__device__ __forceinline__ double vadv_zdis(const WP& wp, const double* rdz, const double* rdzs, int k, int mkmin,
                                           int mkmax, double dt, double hdt2, double sdt3) {
  if (k == mkmin) {
    const double w0 = vadv_wh(wp, mkmin, mkmin, mkmax), wpp = vadv_wh(wp, mkmin + 1, mkmin, mkmax);
    return __fma_rn(-hdt2 * w0, (wpp - w0) * rdz[mkmin], dt * w0);
  }
  const double wm = vadv_wh(wp, k - 1, mkmin, mkmax);
  const double w0 = vadv_wh(wp, k, mkmin, mkmax);
  const double wpp = vadv_wh(wp, k + 1, mkmin, mkmax);
  const double r = (wpp - wm) * rdzs[k];
  const double c = 2.0 * rdzs[k] * __fma_rn(wpp - w0, rdz[k], -(w0 - wm) * rdz[k - 1]);
  const double t3 = sdt3 * w0 * __fma_rn(w0, c, r * r);
  return __fma_rn(-hdt2 * w0, r, __fma_rn(dt, w0, t3));
}

}  // namespace nsw6
