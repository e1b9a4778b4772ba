// Per-cell NSW6 physics (device), FP64.
//
// One call evaluates, for one interior cell, what the reference computes in
// several whole-field passes: negative_filter (mod_mp_nsw6.cpp:1750-1832),
// saturation vapour pressure and mixing ratio (mod_satadjust.cpp:80-160,
// mod_mp_nsw6.cpp:686-690), Bergeron_param (mod_mp_nsw6.cpp:1834-1890), the
// TagBigLoop process rates (mod_mp_nsw6.cpp:760-1594) and the cell updates
// TagUpdateRHOGQ/RHOGE/MassConc/TEM (mod_mp_nsw6.cpp:692-744).  Expressions
// keep the reference's evaluation order; integer powers are products.
#pragma once

#include "nsw6_common.cuh"

namespace nsw6 {

__constant__ double c_a1_tab[32] = {
    0.0001E-7, 0.7939E-7, 0.7841E-6, 0.3369E-5, 0.4336E-5, 0.5285E-5, 0.3728E-5, 0.1852E-5,
    0.2991E-6, 0.4248E-6, 0.7434E-6, 0.1812E-5, 0.4394E-5, 0.9145E-5, 0.1725E-4, 0.3348E-4,
    0.1725E-4, 0.9175E-5, 0.4412E-5, 0.2252E-5, 0.9115E-6, 0.4876E-6, 0.3473E-6, 0.4758E-6,
    0.6306E-6, 0.8573E-6, 0.7868E-6, 0.7192E-6, 0.6513E-6, 0.5956E-6, 0.5333E-6, 0.4834E-6};
__constant__ double c_a2_tab[32] = {
    0.0100, 0.4006, 0.4831, 0.5320, 0.5307, 0.5319, 0.5249, 0.4888, 0.3849, 0.4047, 0.4318,
    0.4771, 0.5183, 0.5463, 0.5651, 0.5813, 0.5655, 0.5478, 0.5203, 0.4906, 0.4447, 0.4126,
    0.3960, 0.4149, 0.4320, 0.4506, 0.4483, 0.4460, 0.4433, 0.4413, 0.4382, 0.4361};

struct CellIn {
  double rhog, rhoge_unused, tem, gsgam2, q0;
  double rhogq[6];
};

struct CellOut {
  double rhog, rhoge, tem;
  double rhogq[6];
  double q[6];
  double Vt[4];  // QR QI QS QG
  double rceff, rceff_cld, rctop, tctop;
};

// Reference constant values that do not depend on the tunable parameters.
constexpr double kEiw = 1.0, kErw = 1.0, kEsw = 1.0, kEgw = 1.0, kEri = 1.0, kEgi = 0.0;
constexpr double kEsr = 1.0, kEgr = 1.0;
constexpr double kGAM = 1.0, kGAM_2 = 1.0, kGAM_3 = 2.0;
constexpr double kF1r = 0.78, kF2r = 0.27, kF1s = 0.65, kF2s = 0.39, kF1g = 0.78, kF2g = 0.27;
constexpr double kVti50 = 1.0;
constexpr double kSwRoh = 1.0, kSwExpice = 1.0, kSwKK = 1.0, kSwConstVti = 0.0;
constexpr double kGammaGaut = 90.E-3, kQscrtGaut = 6.E-4, kBetaGaut = 0.0;

__device__ __forceinline__ double roh_moment(const Consts& C, const double cat[4], const double cbt[4], double nm,
                                             double logX, double zerosw) {
  const double loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  const double b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  return kSwRoh * exp(C.ln10 * loga_) * exp(logX * b_) * (1.0 - zerosw);
}

__device__ __forceinline__ void nsw6_cell(const Consts& C, double dt, const CellIn& in, CellOut& o) {
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
  const double dens = rhog / in.gsgam2;
  double qn[6];
  qn[0] = in.q0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qn[n] = rq[n] / rhog;
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
  const double rtem = 1.0 / (dmax(temp, TEM_MIN));
  const double psatl = PSAT0 * exp(C.LovR_liq * (C.RTEM00 - rtem));
  const double psati = PSAT0 * exp(C.LovR_ice * (C.RTEM00 - rtem));
  const double qsatl = psatl / (dens * RVAP * temp);
  const double qsati = psati / (dens * RVAP * temp);

  // ---- Bergeron_param
  double a1, a2, ma2;
  {
    const double temc_b = dmin(dmax(temp - TEM00, -30.99), 0.0);
    const int itemc = (int)(-temc_b);
    const double fact = -(temc_b + (double)(itemc - 1));
    const double v1 = (1.0 - fact) * c_a1_tab[itemc] + (fact)*c_a1_tab[itemc + 1];
    a2 = (1.0 - fact) * c_a2_tab[itemc] + (fact)*c_a2_tab[itemc + 1];
    ma2 = 1.0 - a2;
    a1 = v1 * pow(1.0E-3, ma2);
  }
  const double Nc = C.Nc_def;

  // ---- TagBigLoop, mod_mp_nsw6.cpp:902-1594
  const double qv = dmax(qn[0], 0.0), qc = dmax(qn[1], 0.0), qr = dmax(qn[2], 0.0);
  const double qi = dmax(qn[3], 0.0), qs = dmax(qn[4], 0.0), qg = dmax(qn[5], 0.0);
  const double Sliq = qv / (dmax(qsatl, EPS));
  const double Sice = qv / (dmax(qsati, EPS));
  const double Rdens = 1.0 / dens;
  const double rho_fact = sqrt(DENS00 * Rdens);
  const double temc = temp - TEM00;
  const double delta1 = (0.5 + copysign(0.5, qr - 1.0E-4));
  const double delta2 = (0.5 + copysign(0.5, 1.0E-4 - qr)) * (0.5 + copysign(0.5, 1.0E-4 - qs));
  const double spsati = 0.5 + copysign(0.5, Sice - 1.0);
  const double iceflg = 0.5 - copysign(0.5, temc);
  const double dqv_dt = qv / dt, dqc_dt = qc / dt, dqr_dt = qr / dt;
  const double dqi_dt = qi / dt, dqs_dt = qs / dt, dqg_dt = qg / dt;
  const double sw_bergeron =
      (0.5 + copysign(0.5, temc + 30.0)) * (0.5 + copysign(0.5, 0.0 - temc)) * (1.0 - kSwExpice);

  double zerosw = 0.5 - copysign(0.5, qr - 1.0E-12);
  const double RLMDr = sqrt(sqrt(dens * qr / (C.Ar * C.N0r * C.GAM_1br) + zerosw)) * (1.0 - zerosw);
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

  zerosw = 0.5 - copysign(0.5, qs - 1.0E-12);
  const double RLMDs = sqrt(sqrt(dens * qs / (C.As * C.N0s * C.GAM_1bs) + zerosw)) * (1.0 - zerosw);
  const double RLMDs_ds = sqrt(sqrt(RLMDs));
  const double RLMDs_2 = RLMDs * RLMDs;
  const double RLMDs_3 = RLMDs_2 * RLMDs;
  const double RLMDs_1bs = RLMDs_2 * RLMDs_2;
  const double RLMDs_2bs = RLMDs_1bs * RLMDs;
  const double RLMDs_3bs = RLMDs_3 * RLMDs_3;
  const double RLMDs_3ds = RLMDs_3 * RLMDs_ds;
  const double RLMDs_5ds = RLMDs_2bs * RLMDs_ds;
  double MOMs_0 = C.N0s * kGAM * RLMDs;
  double MOMs_1 = C.N0s * kGAM_2 * RLMDs_2;
  double MOMs_2 = C.N0s * kGAM_3 * RLMDs_3;
  double MOMs_0bs = C.N0s * C.GAM_1bs * RLMDs_1bs;
  double MOMs_1bs = C.N0s * C.GAM_2bs * RLMDs_2bs;
  double MOMs_2bs = C.N0s * C.GAM_3bs * RLMDs_3bs;
  double MOMs_2ds = C.N0s * C.GAM_3ds * RLMDs_3ds;
  double MOMs_5ds_h = C.N0s * C.GAM_5ds_h * sqrt(RLMDs_5ds);
  double RMOMs_Vt = C.GAM_1bsds / C.GAM_1bs * RLMDs_ds;

  // Roh and Satoh (2014) moments, :994-1057; log(Xs2 + zerosw) is shared.
  const double Xs2 = dens * qs / C.As;
  zerosw = 0.5 - copysign(0.5, Xs2 - 1.0E-12);
  const double tems = dmin(-0.1, temc);
  double cat[4], cbt[4];
  cat[0] = C.coef_a[0] + tems * (C.coef_a[1] + tems * (C.coef_a[4] + tems * C.coef_a[8]));
  cat[1] = C.coef_a[2] + tems * (C.coef_a[3] + tems * C.coef_a[6]);
  cat[2] = C.coef_a[5] + tems * C.coef_a[7];
  cat[3] = C.coef_a[9];
  cbt[0] = C.coef_b[0] + tems * (C.coef_b[1] + tems * (C.coef_b[4] + tems * C.coef_b[8]));
  cbt[1] = C.coef_b[2] + tems * (C.coef_b[3] + tems * C.coef_b[6]);
  cbt[2] = C.coef_b[5] + tems * C.coef_b[7];
  cbt[3] = C.coef_b[9];
  const double logX = log(Xs2 + zerosw);
  MOMs_0 = kSwRoh * exp(C.ln10 * cat[0]) * exp(logX * cbt[0]) * (1.0 - zerosw) + (1.0 - kSwRoh) * MOMs_0;
  MOMs_1 = roh_moment(C, cat, cbt, 1.0, logX, zerosw) + (1.0 - kSwRoh) * MOMs_1;
  MOMs_2 = kSwRoh * Xs2 + (1.0 - kSwRoh) * MOMs_2;
  MOMs_0bs = roh_moment(C, cat, cbt, 2.0, logX, zerosw) + (1.0 - kSwRoh) * MOMs_0bs;
  MOMs_1bs = roh_moment(C, cat, cbt, 3.0, logX, zerosw) + (1.0 - kSwRoh) * MOMs_1bs;
  MOMs_2bs = roh_moment(C, cat, cbt, 4.0, logX, zerosw) + (1.0 - kSwRoh) * MOMs_2bs;
  const double m225 = roh_moment(C, cat, cbt, 2.25, logX, zerosw);
  MOMs_2ds = m225 + (1.0 - kSwRoh) * MOMs_2ds;
  MOMs_5ds_h = roh_moment(C, cat, cbt, 1.625, logX, zerosw) + (1.0 - kSwRoh) * MOMs_5ds_h;
  RMOMs_Vt = m225 / (MOMs_0bs + zerosw) + (1.0 - kSwRoh) * RMOMs_Vt;

  zerosw = 0.5 - copysign(0.5, qg - 1.0E-12);
  const double RLMDg = sqrt(sqrt(dens * qg / (C.Ag * C.N0g * C.GAM_1bg) + zerosw)) * (1.0 - zerosw);
  const double RLMDg_dg = sqrt(RLMDg);
  const double RLMDg_2 = RLMDg * RLMDg;
  const double RLMDg_3 = RLMDg_2 * RLMDg;
  const double RLMDg_3dg = RLMDg_3 * RLMDg_dg;
  const double RLMDg_5dg = RLMDg_3 * RLMDg_2 * RLMDg_dg;

  // terminal velocity, :1072-1078
  zerosw = 0.5 - copysign(0.5, qi - 1.0E-8);
  const double Vti = (1.0 - kSwConstVti) * (-3.29) * exp(log(dens * qi + zerosw) * 0.16) * (1.0 - zerosw) +
                     (kSwConstVti) * (-UNDEF);
  const double Vtr = -C.Cr * rho_fact * C.GAM_1brdr / C.GAM_1br * RLMDr_dr;
  const double Vts = -C.Cs * rho_fact * RMOMs_Vt;
  const double Vtg = -C.Cg * rho_fact * C.GAM_1bgdg / C.GAM_1bg * RLMDg_dg;

  // nucleation, :1080-1085
  const double Ni0 = dmax(exp(-0.1 * temc), 1.0) * 1000.0;
  const double Qi0 = C.ice_nuc * exp(log(Ni0) * 1.33) * Rdens;
  double Pigen = dmax(dmin(Qi0 - qi, qv - qsati), 0.0) / dt;

  // accretion, :1087-1145
  const double Esi_mod = dmin(C.Esi, C.Esi * exp(C.gamma_sacr * temc));
  const double Egs_mod = dmin(C.Egs, C.Egs * exp(C.gamma_gacs * temc));
  zerosw = 0.5 - copysign(0.5, qc * qr - 1.0E-12);
  const double Pracw_kk = 67.0 * exp(log(qc * qr + zerosw) * 1.15) * (1.0 - zerosw);
  const double Pracw_orig = qc * 0.25 * PI * kErw * C.N0r * C.Cr * C.GAM_3dr * RLMDr_3dr * rho_fact;
  double Pracw = (1.0 - kSwKK) * Pracw_orig + (kSwKK)*Pracw_kk;
  double Psacw = qc * 0.25 * PI * kEsw * C.Cs * MOMs_2ds * rho_fact;
  double Pgacw = qc * 0.25 * PI * kEgw * C.N0g * C.Cg * C.GAM_3dg * RLMDg_3dg * rho_fact;
  double Praci = qi * 0.25 * PI * kEri * C.N0r * C.Cr * C.GAM_3dr * RLMDr_3dr * rho_fact;
  double Psaci = qi * 0.25 * PI * Esi_mod * C.Cs * MOMs_2ds * rho_fact;
  double Pgaci = qi * 0.25 * PI * kEgi * C.N0g * C.Cg * C.GAM_3dg * RLMDg_3dg * rho_fact;
  double Piacr = qi * C.Ar / C.mi * 0.25 * PI * kEri * C.N0r * C.Cr * C.GAM_6dr * RLMDr_6dr * rho_fact;
  double Psacr = C.Ar * 0.25 * PI * Rdens * kEsr * C.N0r * fabs(Vtr - Vts) *
                 (C.GAM_1br * RLMDr_1br * MOMs_2 + 2.0 * C.GAM_2br * RLMDr_2br * MOMs_1 +
                  C.GAM_3br * RLMDr_3br * MOMs_0);
  double Pgacr = C.Ar * 0.25 * PI * Rdens * kEgr * C.N0g * C.N0r * fabs(Vtg - Vtr) *
                 (C.GAM_1br * RLMDr_1br * kGAM_3 * RLMDg_3 + 2.0 * C.GAM_2br * RLMDr_2br * kGAM_2 * RLMDg_2 +
                  C.GAM_3br * RLMDr_3br * kGAM * RLMDg);
  double Pracs = C.As * 0.25 * PI * Rdens * kEsr * C.N0r * fabs(Vtr - Vts) *
                 (MOMs_0bs * kGAM_3 * RLMDr_3 + 2.0 * MOMs_1bs * kGAM_2 * RLMDr_2 + MOMs_2bs * kGAM * RLMDr);
  double Pgacs = C.As * 0.25 * PI * Rdens * Egs_mod * C.N0g * fabs(Vtg - Vts) *
                 (MOMs_0bs * kGAM_3 * RLMDg_3 + 2.0 * MOMs_1bs * kGAM_2 * RLMDg_2 + MOMs_2bs * kGAM * RLMDg);

  // autoconversion, :1147-1172 (only the second Praut_kk assignment is live)
  const double rhoqc = dens * qc * 1000.0;
  const double Dc = C.Dc_berry;  // 0.146 - 5.964E-2 * log(Nc / 2000.0) with Nc = Nc_def
  const double Praut_berry = Rdens * 1.67E-5 * rhoqc * rhoqc / (5.0 + 3.66E-2 * Nc / (Dc * rhoqc + EPS));
  const double Praut_kk = C.kk_aut * pow(qc, 2.47) * C.pow_Nc_m179;
  double Praut = (1.0 - kSwKK) * Praut_berry + kSwKK * Praut_kk;
  const double betai = dmin(C.beta_saut, C.beta_saut * exp(C.gamma_saut * temc));
  double Psaut = dmax(betai * (qi - C.qicrt_saut), 0.0);
  const double betas = dmin(kBetaGaut, kBetaGaut * exp(kGammaGaut * temc));
  double Pgaut = dmax(betas * (qs - kQscrtGaut), 0.0);

  // evaporation, sublimation, melting and freezing, :1174-1247
  const double Ka = (2.428E-2 + 7.47E-5 * temc);
  const double Kd = (2.222E-5 + 1.37E-7 * temc) * PSTD / pre;
  const double Nu = (1.718E-5 + 5.28E-8 * temc) * Rdens;
  const double Glv = 1.0 / (LHV0 / (Ka * temp) * (LHV0 / (RVAP * temp) - 1.0) + 1.0 / (Kd * dens * qsatl));
  const double Giv = 1.0 / (LHS0 / (Ka * temp) * (LHS0 / (RVAP * temp) - 1.0) + 1.0 / (Kd * dens * qsati));
  const double Gil = 1.0 / (LHF0 / (Ka * temc));
  const double ventr = kF1r * kGAM_2 * RLMDr_2 + kF2r * sqrt(C.Cr * rho_fact / Nu * RLMDr_5dr) * C.GAM_5dr_h;
  double Prevp = 2.0 * PI * Rdens * C.N0r * (1.0 - dmin(Sliq, 1.0)) * Glv * ventr;
  const double rhoqi = dmax(dens * qi, EPS);
  const double XNi = dmin(dmax(5.38E+7 * exp(log(rhoqi) * 0.75), 1.0E+3), 1.0E+6);
  const double XMi = rhoqi / XNi;
  const double Di = dmin(C.Di_a * sqrt(XMi), C.Di_max);
  double tmp = 4.0 * Di * XNi * Rdens * (Sice - 1.0) * Giv;
  double Pidep = (spsati) * (tmp);
  double Pisub = (1.0 - spsati) * (-tmp);
  double sw = (0.5 - copysign(0.5, temc + 40.0));
  double Pihom = sw * qc / dt;
  sw = (0.5 + copysign(0.5, temc + 40.0)) * (0.5 - copysign(0.5, temc));
  const double efrz = exp(-C.A_frz * temc) - 1.0;
  double Pihtr = sw * (dens / DWATR * (qc * qc) / (C.Nc_ihtr * 1.0E+6)) * C.B_frz * efrz;
  sw = (0.5 + copysign(0.5, temc));
  double Pimlt = sw * qi / dt;
  const double vents = kF1s * MOMs_1 + kF2s * sqrt(C.Cs * rho_fact / Nu) * MOMs_5ds_h;
  tmp = 2.0 * PI * Rdens * (Sice - 1.0) * Giv * vents;
  double Psdep = (spsati) * (tmp);
  double Pssub = (1.0 - spsati) * (-tmp);
  double Psmlt = 2.0 * PI * Rdens * Gil * vents + CL * temc / LHF0 * (Psacw + Psacr);
  Psmlt = dmax(Psmlt, 0.0);
  const double ventg = kF1g * kGAM_2 * RLMDg_2 + kF2g * sqrt(C.Cg * rho_fact / Nu * RLMDg_5dg) * C.GAM_5dg_h;
  tmp = 2.0 * PI * Rdens * C.N0g * (Sice - 1.0) * Giv * ventg;
  double Pgdep = (spsati) * (tmp);
  double Pgsub = (1.0 - spsati) * (-tmp);
  double Pgmlt = 2.0 * PI * Rdens * C.N0g * Gil * ventg + CL * temc / LHF0 * (Pgacw + Pgacr);
  Pgmlt = dmax(Pgmlt, 0.0);
  double Pgfrz = 2.0 * PI * Rdens * C.N0r * 60.0 * C.B_frz * C.Ar * efrz * RLMDr_7;
  const double dt1 = (exp(C.log_mi50 * ma2) - exp(C.log_mi40 * ma2)) / (a1 * ma2);
  const double Ni50 = qi * dt / (C.mi50 * dt1);
  double Psfw = Ni50 * (a1 * pow(C.mi50, a2) + PI * kEiw * dens * qc * C.Ri50 * C.Ri50 * kVti50);
  double Psfi = qi / dt1;

  // limiters, :1249-1296
  Pigen = dmin(Pigen, dqv_dt) * (iceflg)*kSwExpice;
  Pidep = dmin(Pidep, dqv_dt) * (iceflg)*kSwExpice;
  Psdep = dmin(Psdep, dqv_dt) * (iceflg);
  Pgdep = dmin(Pgdep, dqv_dt) * (iceflg);
  Pracw = Pracw + Psacw * (1.0 - iceflg) + Pgacw * (1.0 - iceflg);
  Praut = dmin(Praut, dqc_dt);
  Pracw = dmin(Pracw, dqc_dt);
  Pihom = dmin(Pihom, dqc_dt) * (iceflg)*kSwExpice;
  Pihtr = dmin(Pihtr, dqc_dt) * (iceflg)*kSwExpice;
  Psacw = dmin(Psacw, dqc_dt) * (iceflg);
  Psfw = dmin(Psfw, dqc_dt) * (iceflg)*sw_bergeron;
  Pgacw = dmin(Pgacw, dqc_dt) * (iceflg);
  Prevp = dmin(Prevp, dqr_dt);
  Piacr = dmin(Piacr, dqr_dt) * (iceflg);
  Psacr = dmin(Psacr, dqr_dt) * (iceflg);
  Pgacr = dmin(Pgacr, dqr_dt) * (iceflg);
  Pgfrz = dmin(Pgfrz, dqr_dt) * (iceflg);
  Pisub = dmin(Pisub, dqi_dt) * (iceflg)*kSwExpice;
  Pimlt = dmin(Pimlt, dqi_dt) * (1.0 - iceflg) * kSwExpice;
  Psaut = dmin(Psaut, dqi_dt) * (iceflg);
  Praci = dmin(Praci, dqi_dt) * (iceflg);
  Psaci = dmin(Psaci, dqi_dt) * (iceflg);
  Psfi = dmin(Psfi, dqi_dt) * (iceflg)*sw_bergeron;
  Pgaci = dmin(Pgaci, dqi_dt) * (iceflg);
  Pssub = dmin(Pssub, dqs_dt) * (iceflg);
  Psmlt = dmin(Psmlt, dqs_dt) * (1.0 - iceflg);
  Pgaut = dmin(Pgaut, dqs_dt) * (iceflg);
  Pracs = dmin(Pracs, dqs_dt) * (iceflg);
  Pgacs = dmin(Pgacs, dqs_dt);
  Pgsub = dmin(Pgsub, dqg_dt) * (iceflg);
  Pgmlt = dmin(Pgmlt, dqg_dt) * (1.0 - iceflg);
  double Piacr_s = (1.0 - delta1) * Piacr;
  double Piacr_g = (delta1)*Piacr;
  double Praci_s = (1.0 - delta1) * Praci;
  double Praci_g = (delta1)*Praci;
  double Psacr_s = (delta2)*Psacr;
  double Psacr_g = (1.0 - delta2) * Psacr;
  Pracs = (1.0 - delta2) * Pracs;

  double net, fac, fac_sw;
  // [QC] :1298-1320
  net = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Psfw - Pgacw;
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-dqc_dt / (net - fac_sw), 1.0);
  Pimlt *= fac; Praut *= fac; Pracw *= fac; Pihom *= fac; Pihtr *= fac; Psacw *= fac; Psfw *= fac; Pgacw *= fac;
  // [QI] :1322-1354
  net = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Psfi - Praci_g - Pgaci;
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-dqi_dt / (net - fac_sw), 1.0);
  Pigen *= fac; Pidep *= fac; Pihom *= fac; Pihtr *= fac; Pisub *= fac; Pimlt *= fac; Psaut *= fac;
  Praci_s *= fac; Psaci *= fac; Psfi *= fac; Praci_g *= fac; Pgaci *= fac;
  // [QR] :1357-1385
  net = +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz;
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-dqr_dt / (net - fac_sw), 1.0);
  Praut *= fac; Pracw *= fac; Psmlt *= fac; Pgmlt *= fac; Prevp *= fac; Piacr_s *= fac; Psacr_s *= fac;
  Piacr_g *= fac; Psacr_g *= fac; Pgacr *= fac; Pgfrz *= fac;
  // [QV] :1387-1407
  net = +Prevp + Pisub + Pssub + Pgsub - Pigen - Pidep - Psdep - Pgdep;
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-dqv_dt / (net - fac_sw), 1.0);
  Prevp *= fac; Pisub *= fac; Pssub *= fac; Pgsub *= fac; Pigen *= fac; Pidep *= fac; Psdep *= fac; Pgdep *= fac;
  // [QS] :1409-1443
  net = +Psdep + Psacw + Psfw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci + Psfi - Pssub - Psmlt - Pgaut - Pracs -
        Pgacs;
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-dqs_dt / (net - fac_sw), 1.0);
  Psdep *= fac; Psacw *= fac; Psfw *= fac; Piacr_s *= fac; Psacr_s *= fac; Psaut *= fac; Praci_s *= fac;
  Psaci *= fac; Psfi *= fac; Pssub *= fac; Psmlt *= fac; Pgaut *= fac; Pracs *= fac; Pgacs *= fac;
  // [QG] :1445-1477
  net = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pgaci + Pgaut + Pracs + Pgacs - Pgsub - Pgmlt;
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-dqg_dt / (net - fac_sw), 1.0);
  Pgdep *= fac; Pgacw *= fac; Piacr_g *= fac; Psacr_g *= fac; Pgacr *= fac; Pgfrz *= fac; Praci_g *= fac;
  Pgaci *= fac; Pgaut *= fac; Pracs *= fac; Pgacs *= fac; Pgsub *= fac; Pgmlt *= fac;

  // tendencies, :1479-1559
  double qc_t = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Psfw - Pgacw;
  double qr_t = +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz;
  double qi_t = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Psfi - Praci_g - Pgaci;
  double qs_t = +Psdep + Psacw + Psfw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci + Psfi - Pssub - Psmlt - Pgaut -
                Pracs - Pgacs;
  double qg_t =
      +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pgaci + Pgaut + Pracs + Pgacs - Pgsub - Pgmlt;
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
  o.Vt[0] = Vtr;
  o.Vt[1] = Vti;
  o.Vt[2] = Vts;
  o.Vt[3] = Vtg;

  // effective radius and cloud top, :1566-1592
  {
    const double r2_min = 1.0E-10, q_min = 1.0E-5;
    const double xf_qc = rhoqc / Nc * 1.0E-9;
    const double rf_qc = pow((C.coef_xf * xf_qc + EPS), 0.33333333);
    const double r2_qc = C.coef_dgam * (rf_qc * rf_qc) * (Nc * 1.0E+6);
    const double r2_qr = 0.25 * C.N0r * kGAM_3 * RLMDr_3;
    const double r3_qc = C.coef_xf * dens * qc;
    const double r3_qr = C.coef_xf * dens * qr;
    zerosw = 0.5 - copysign(0.5, (r2_qc + r2_qr) - r2_min);
    o.rceff = (r3_qc + r3_qr) / (r2_qc + r2_qr + zerosw) * (1.0 - zerosw);
    sw = (0.5 + copysign(0.5, (qc + qr) - q_min)) * zerosw;
    o.rctop = (sw)*o.rceff + (1.0 - sw) * UNDEF;
    o.tctop = (sw)*temp + (1.0 - sw) * UNDEF;
    zerosw = 0.5 - copysign(0.5, r2_qc - r2_min);
    o.rceff_cld = r3_qc / (r2_qc + zerosw) * (1.0 - zerosw);
  }

  // ---- TagUpdateRHOGQ / RHOGE / MassConc / TEM, mod_mp_nsw6.cpp:692-744
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] += drq[n];
  rhoge = rhoge - LHV0 * drq[I_QV] + LHF0 * drq[I_QI] + LHF0 * drq[I_QS] + LHF0 * drq[I_QG];
  o.q[0] = qn[0];
#pragma unroll
  for (int n = 1; n <= 5; ++n) o.q[n] = rq[n] / rhog;
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
// (mod_vadv1d.cpp:284-302).
template <class WP>
__device__ __forceinline__ double vadv_zdis(const WP& wp, const double* dz, int k, int mkmin, int mkmax, double dt,
                                           double dt2, double dt3) {
  if (k == mkmin) {
    const double w0 = vadv_wh(wp, mkmin, mkmin, mkmax), wpp = vadv_wh(wp, mkmin + 1, mkmin, mkmax);
    return dt * w0 - dt2 * w0 * (wpp - w0) / dz[mkmin] / 2.0;
  }
  const double wm = vadv_wh(wp, k - 1, mkmin, mkmax);
  const double w0 = vadv_wh(wp, k, mkmin, mkmax);
  const double wpp = vadv_wh(wp, k + 1, mkmin, mkmax);
  const double dzs = dz[k - 1] + dz[k];
  const double r = (wpp - wm) / dzs;
  return dt * w0 - dt2 * w0 * (wpp - wm) / dzs / 2.0 +
         dt3 * w0 * (r * r + w0 * (((wpp - w0) / dz[k] - (w0 - wm) / dz[k - 1]) / dzs * 2.0)) / 6.0;
}

}  // namespace nsw6
