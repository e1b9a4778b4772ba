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
//
// With OPT = true the same function also evaluates the branches that the
// scheme switches select (ConstsT::opt_*, nsw6_options): the classic snow
// moments (:975-992), the Bergeron terms with Bergeron_param
// (:1239-1247, :1834-1890), Berry autoconversion and the original accretion
// (:1091-1099, :1145-1160), the graupel accretion of ice and snow (:1116,
// :1136-1140), the ice fall speed (:1073-1075) and the cloud number from the
// CCN input (:676-679); each term enters the limiters and tendencies at the
// reference's position.
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

template <class D>
struct CellInT {
  D rhog, tem, gsgam2, q0;
  D rhogq[6];
  D unccn;   // read only with the aerosol-indirect switch
};

template <class D>
struct CellOutT {
  D rhog, rhoge, tem;
  D rhogq[6];
  D q[6];
  D Vtr, Vts, Vtg, Vti;   // Vti only with OPT
  D rceff, rceff_cld, rctop, tctop;
};
using CellIn = CellInT<double>;
using CellOut = CellOutT<double>;

// Scalar helpers overloaded on the precision of the process rates (FP64 in
// the plain path, FP32 in the mixed path).
__device__ __forceinline__ double fmaR(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmaR(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double sqrtR(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrtR(float x) { return sqrtf(x); }
__device__ __forceinline__ double fabsR(double x) { return fabs(x); }
__device__ __forceinline__ float fabsR(float x) { return fabsf(x); }
__device__ __forceinline__ double val_of(double x) { return x; }   // the value of a scalar (its
__device__ __forceinline__ float val_of(float x) { return x; }     // derivative types add theirs)
__device__ __forceinline__ float dmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float dmax(float a, float b) { return (a < b) ? b : a; }

// A process rate clamped at zero, max(x, 0) (Kokkos::max as above).  Its
// derivative types (nsw6_ad.cuh) treat the rate as off where x is exactly
// zero: the ice->snow autoconversion max(beta (qi - qicrt), 0) sits there in
// every cell without ice at the reference threshold qicrt = 0, where the ice
// limiters hold the rate at zero on both sides of the threshold.
template <class R>
__device__ __forceinline__ R rate_on(const R& x) { return dmax(x, R(0)); }
// x * f for a switch value f in {0, 1} (the reference's iceflg, delta1,
// delta2, spsati): x, or the zero x * 0 gives (a zero with the sign of x),
// selected without an FP64 multiplication.
__device__ __forceinline__ double sel(bool on, double x) { return on ? x : copysign(0.0, x); }
__device__ __forceinline__ float sel(bool on, float x) { return on ? x : copysignf(0.0f, x); }

// q / dt of the rates: the correctly rounded quotient in FP64 (the reference
// divides), a product with 1/dt in FP32.
__device__ __forceinline__ double per_dt(double q, double dt, double rdt) { return div_rn(q, dt, rdt); }
__device__ __forceinline__ float per_dt(float q, float, float rdt) { return q * rdt; }

// The comparisons of the cell physics with constants and the min / max they
// select: for doubles the integer-pipe forms of nsw6_fpcmp.cuh (an FP64
// comparison takes an FP64-pipe slot, as an FMA does); the other types compare
// natively (FP32 comparisons are cheap, the derivative types compare values).
template <class T>
__device__ __forceinline__ bool is_one(const T& x) { return x == T(1.0); }
template <class T>
__device__ __forceinline__ bool is_nonneg(const T& x) { return x >= T(0.0); }

template <class T>
__device__ __forceinline__ bool lt_z(const T& x) { return x < T(0.0); }
template <class T>
__device__ __forceinline__ bool gt_z(const T& x) { return x > T(0.0); }
template <class T>
__device__ __forceinline__ bool ge_c(const T& x, const T& c) { return x >= c; }
template <class T>
__device__ __forceinline__ bool gt_c(const T& x, const T& c) { return x > c; }
template <class T>
__device__ __forceinline__ bool le_c(const T& x, const T& c) { return x <= c; }
template <class T>
__device__ __forceinline__ bool lt_negc(const T& x, const T& c) { return x < c; }
template <class T>
__device__ __forceinline__ bool lt_c(const T& x, const T& c) { return x < c; }
template <class T>
__device__ __forceinline__ T maxz(const T& x) { return dmax(x, T(0.0)); }
template <class T>
__device__ __forceinline__ bool is_zero(const T& x) { return x == T(0.0); }
__device__ __forceinline__ double rate_on(double x) { return maxz(x); }
template <class T>
__device__ __forceinline__ T maxc(const T& x, const T& c) { return dmax(x, c); }
template <class T>
__device__ __forceinline__ T minc(const T& x, const T& c) { return dmin(x, c); }
template <class T>
__device__ __forceinline__ bool lt_nn(const T& d, const T& p) { return d < p; }
template <class T>
__device__ __forceinline__ T min_nn(const T& p, const T& d) { return dmin(p, d); }
template <class T>
__device__ __forceinline__ bool lt_nd(const T& a, const T& d) { return a < -d; }
template <class T>
__device__ __forceinline__ T max_nd(const T& a, const T& d) { return dmax(a, -d); }

// The liquid saturation test qsum - qsat(T) > EPS of the saturation
// adjustment (mod_satadjust.cpp:771-896), decided in FP32 where its margin
// allows: 1 saturated, 0 not, -1 left to the FP64 test.  Three conversions
// (T, rho, qsum): an FP64 compare or conversion costs as much of the FP64
// pipe as an FMA.  x = LovR (1/T00 - 1/T) is formed as LovR (Tf - T00f) /
// (Tf T00f): the difference is exact, so x carries seven roundings
// (4.2e-7 |x|) and the conversions of T and T00 (LovR u (1/T00 + 1/T) <=
// 7.2e-6 for |x| <= 80, u = 2^-24); with expf's 2 ulp and eight roundings
// after it the FP32 qsat is within 4.2e-5 (relative) of the FP64 one, and
// qsum rounds by u.  So qsum_f > 1.0001 qsat_f means qsum > (1 + 5.7e-5) qsat,
// and with qsat_f >= 1e-11 the FP64 difference exceeds EPS; qsum_f <
// 0.9999 qsat_f means qsum < qsat.  Cells in between and outside those ranges
// (and NaNs) are left to the FP64 test, as the reference computes it.
// lovr_f = float(LovR_liq).
__device__ __forceinline__ int sat_screen_liq(double tem, double rho, double qsum, float lovr_f) {
  const float tf = float(tem);
  const float tcf = (tf < float(TEM_MIN)) ? float(TEM_MIN) : tf;   // float(max(tem, TEM_MIN))
  const float xf = lovr_f * ((tcf - float(TEM00)) / (tcf * float(TEM00)));
  if (!(fabsf(xf) <= 80.0f)) return -1;
  const float qsf = (float(PSAT0) * expf(xf)) / (float(rho) * float(RVAP) * tf);
  if (!(qsf >= 1.0e-11f && qsf <= 1.0e30f)) return -1;
  const float qq = float(qsum);
  if (qq > qsf * 1.0001f) return 1;
  if (qq < qsf * 0.9999f) return 0;
  return -1;
}

// R = double: the plain FP64 step.  R = float (the mixed path): saturation
// values, process rates, limiters, tendencies, fall speeds and effective radii
// in FP32; the negative filter, the tracer and internal-energy budgets
// (rhogq += drhogq, rhoge) and the temperature update stay FP64.
//
// D is the type of the state and budget arithmetic: double in both paths; the
// tangent-linear and adjoint kernels instantiate R = D with their derivative
// types (nsw6_ad.cuh).
template <class M, class R, class D = double, bool OPT = false>
__device__ __forceinline__ void nsw6_cell(const ConstsT<R>& C, const M& mth, double dt, double rdt,
                                          const CellInT<D>& in, CellOutT<D>& o) {
  constexpr bool kMixed = sizeof(R) == sizeof(float);
  const R dtR = R(dt), rdtR = R(rdt);
  // ---- negative_filter, mod_mp_nsw6.cpp:1770-1831
  D rq[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] = in.rhogq[n];
  D diffq = D(0.0);
#pragma unroll
  for (int n = 2; n <= 5; ++n) {
    diffq += rq[n];
    rq[n] = maxz(rq[n]);
  }
#pragma unroll
  for (int n = 2; n <= 5; ++n) diffq -= rq[n];
  rq[I_QV] += diffq;
  diffq = rq[I_QV];
  rq[I_QV] = maxz(rq[I_QV]);
  diffq -= rq[I_QV];
  const D rhog = in.rhog * (1.0 - diffq);
  const D rrhog = 1.0 / rhog;
  D qn[6];
  qn[0] = in.q0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qn[n] = kMixed ? rq[n] * rrhog : div_rn(rq[n], rhog, rrhog);
  const D temp = in.tem;
  D rhoge;
  R pre, densR;
  if constexpr (kMixed) {
    // The internal energy rhog cv T in FP64 with cv = CVdry: under the
    // "SIMPLE" internal energy every CVW is CVdry, so the reference's
    // qd CVdry + sum q CVW is CVdry up to its roundings.  Density and
    // pressure scale FP32 rates only: FP32.
    rhoge = temp * rhog * CVDRY;
    densR = R(rhog) / R(in.gsgam2);
    R qdR = R(1.0);
#pragma unroll
    for (int n = 1; n <= 5; ++n) qdR = qdR - R(qn[n]);
    pre = densR * (qdR * R(RDRY) + R(qn[0]) * R(RVAP)) * R(temp);
  } else {
    const D dens = rhog / in.gsgam2;
    D qd = D(1.0);
#pragma unroll
    for (int n = 1; n <= 5; ++n) qd = qd - qn[n];
    D cv = qd * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cv = cv + qn[n] * CVDRY;
    rhoge = temp * rhog * cv;
    pre = R(dens * (qd * RDRY + qn[0] * RVAP) * temp);
    densR = R(dens);
  }

  // ---- psat / qsat (CPovR = 0 under EIN_TYPE "SIMPLE": the power term is 1)
  const R tempR = R(temp);
  const R rtem = R(1.0) / maxc(tempR, R(TEM_MIN));
  const R psatl = R(PSAT0) * mth.exp(C.LovR_liq * (C.RTEM00 - rtem));
  const R psati = R(PSAT0) * mth.exp(C.LovR_ice * (C.RTEM00 - rtem));
  const R rdrt = R(1.0) / (densR * R(RVAP) * tempR);
  const R qsatl = psatl * rdrt;
  const R qsati = psati * rdrt;

  // ---- TagBigLoop, mod_mp_nsw6.cpp:902-1594
  const R Z = R(0.0), ONE = R(1.0);
  const R qv = maxz(R(qn[0])), qc = maxz(R(qn[1])), qr = maxz(R(qn[2]));
  const R qi = maxz(R(qn[3])), qs = maxz(R(qn[4])), qg = maxz(R(qn[5]));
  const R Sliq = qv / maxc(qsatl, R(EPS));
  const R Sice = qv / maxc(qsati, R(EPS));
  const R Rdens = ONE / densR;
  const R rho_fact = sqrtR(R(DENS00) * Rdens);
  const R temc = tempR - R(TEM00);
  const bool warm = !lt_z(temc);  // iceflg = 0.5 - copysign(0.5, temc) == 0
  const bool d1 = ge_c(qr, R(1.0E-4));                          // delta1
  const bool d2 = le_c(qr, R(1.0E-4)) && le_c(qs, R(1.0E-4));       // delta2
  const bool sps = ge_c(Sice, ONE);                              // spsati
  const R dqv_dt = per_dt(qv, dtR, rdtR), dqc_dt = per_dt(qc, dtR, rdtR), dqr_dt = per_dt(qr, dtR, rdtR);
  const R dqi_dt = per_dt(qi, dtR, rdtR), dqs_dt = per_dt(qs, dtR, rdtR), dqg_dt = per_dt(qg, dtR, rdtR);

  // The blocks of a species that is absent are skipped: every quantity they
  // would compute is then exactly zero (the reference evaluates them with a
  // zero slope parameter or moment), which is what the initial values hold.
  // The cell kernel groups cells by species so that whole warps skip them.

  // rain slope parameter, :953-967
  const bool rain = ge_c(qr, R(1.0E-12));
  R RLMDr = Z, RLMDr_dr = Z, RLMDr_2 = Z, RLMDr_3 = Z, RLMDr_1br = Z, RLMDr_2br = Z, RLMDr_3br = Z, RLMDr_7 = Z;
  R RLMDr_3dr = Z, RLMDr_5dr = Z, RLMDr_6dr = Z;
  if (rain) {
    RLMDr = sqrtR(sqrtR(densR * qr * C.K_rlmdr));
    RLMDr_dr = sqrtR(RLMDr);
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

  // Roh and Satoh (2014) snow moments, :994-1057.  Each moment is
  // 10^loga * Xs2^b = exp(ln10 * loga + log(Xs2) * b), with loga and b
  // polynomials in tems whose coefficients per moment are folded on the host.
  const R Xs2 = densR * qs * C.rAs;
  const bool roh = !OPT || C.opt_roh != Z;
  const bool snow = roh && ge_c(Xs2, R(1.0E-12));
  R mom[7] = {Z, Z, Z, Z, Z, Z, Z};  // MOMs_0, _1, _0bs, _1bs, _2bs, _2ds (= nm 2.25), _5ds_h
  R RMOMs_Vt = Z;
  R MOMs_2 = Xs2;
  if constexpr (OPT) {
    // classic moments of the snow size distribution, :975-992, with
    // RLMDs = (dens qs / (As N0s GAM_1bs))^(1/4) and integer powers as products
    if (!roh) {
      MOMs_2 = Z;
      if (ge_c(qs, R(1.0E-12))) {
        const R s1 = sqrtR(sqrtR(densR * qs * C.K_rlmds));
        const R ds = sqrtR(sqrtR(s1));
        const R s2 = s1 * s1, s3 = s2 * s1, s4 = s2 * s2, s5 = s4 * s1, s6 = s3 * s3;
        mom[0] = C.K_m0 * s1;
        mom[1] = C.K_m1 * s2;
        MOMs_2 = C.K_m2 * s3;
        mom[2] = C.K_m0bs * s4;
        mom[3] = C.K_m1bs * s5;
        mom[4] = C.K_m2bs * s6;
        mom[5] = C.K_m2ds * (s3 * ds);
        mom[6] = C.K_m5dsh * sqrtR(s5 * ds);
        RMOMs_Vt = C.K_rmomvt * ds;
      }
    }
  }
  if (snow) {
    const R tems = lt_negc(temc, R(-0.1)) ? temc : R(-0.1);   // min(-0.1, temc)
    const R logX = mth.log(Xs2);
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const R* a = C.roh_a + 4 * i;
      const R* b = C.roh_b + 4 * i;
      const R la = fmaR(fmaR(fmaR(a[3], tems, a[2]), tems, a[1]), tems, a[0]);
      const R lb = fmaR(fmaR(fmaR(b[3], tems, b[2]), tems, b[1]), tems, b[0]);
      mom[i] = mth.exp(fmaR(logX, lb, la));
    }
    RMOMs_Vt = mom[5] / mom[2];
  }
  const R MOMs_0 = mom[0], MOMs_1 = mom[1];
  const R MOMs_0bs = mom[2], MOMs_1bs = mom[3], MOMs_2bs = mom[4], MOMs_2ds = mom[5];
  const R MOMs_5ds_h = mom[6];

  // graupel slope parameter, :1059-1066
  const bool graupel = ge_c(qg, R(1.0E-12));
  R RLMDg = Z, RLMDg_dg = Z, RLMDg_2 = Z, RLMDg_3 = Z, RLMDg_3dg = Z, RLMDg_5dg = Z;
  if (graupel) {
    RLMDg = sqrtR(sqrtR(densR * qg * C.K_rlmdg));
    RLMDg_dg = sqrtR(RLMDg);
    RLMDg_2 = RLMDg * RLMDg;
    RLMDg_3 = RLMDg_2 * RLMDg;
    RLMDg_3dg = RLMDg_3 * RLMDg_dg;
    RLMDg_5dg = RLMDg_3 * RLMDg_2 * RLMDg_dg;
  }

  // terminal velocity, :1072-1078
  const R Vtr = C.K_vtr * rho_fact * RLMDr_dr;
  const R Vts = C.K_vts * rho_fact * RMOMs_Vt;
  const R Vtg = C.K_vtg * rho_fact * RLMDg_dg;
  R Vti = Z;
  if constexpr (OPT) {
    // :1073-1075 with sw_constVti = 0 (CONST_Vti is UNDEF)
    if (C.opt_qised != Z && qi >= R(1.0E-8)) Vti = R(-3.29) * mth.exp(mth.log(densR * qi) * R(0.16));
  }
  // cloud number (TagAerosolT / TagAerosolF, :676-684)
  R Nc = C.Nc_def;
  if constexpr (OPT) {
    if (C.opt_indir != Z) Nc = dmax(R(in.unccn) * R(1.0E-6), C.Nc_def);
  }

  // nucleation, :1080-1085: Ni0 = max(exp(-0.1 temc), 1) * 1000 and
  // Qi0 = ice_nuc * Ni0^1.33 / dens, with log(Ni0) = ln 1000 + max(-0.1 temc, 0)
  const R Qi0 = C.ice_nuc * mth.exp(R(1.33) * (C.ln1000 + maxz(R(-0.1) * temc))) * Rdens;
  R Pigen = maxz(dmin(Qi0 - qi, qv - qsati)) * rdtR;

  // accretion, :1087-1145
  // Esi_mod and betai, :1089, :1162: min(E, E exp(0.06 temc)) is E when temc >= 0
  // (exp >= 1 there) and E >= 0; both use the same exponential when
  // gamma_sacr == gamma_saut (both 6e-2 in this configuration).
  R Esi_mod = C.Esi, betai = C.beta_saut;
  if (!(warm && is_nonneg(C.Esi) && is_nonneg(C.beta_saut))) {
    const R eg = mth.exp(C.gamma_sacr * temc);
    const R eb = (C.gamma_saut == C.gamma_sacr) ? eg : mth.exp(C.gamma_saut * temc);
    Esi_mod = dmin(C.Esi, C.Esi * eg);
    betai = dmin(C.beta_saut, C.beta_saut * eb);
  }
  const bool kk = !OPT || C.opt_kk != Z;
  const R fr = rho_fact;
  const R qcqr = qc * qr;
  R Pracw = Z;
  if (kk) {
    if (ge_c(qcqr, R(1.0E-12))) Pracw = R(67.0) * mth.pow(qcqr, R(1.15));
  } else {
    Pracw = qc * C.K_raci * RLMDr_3dr * fr;   // Pracw_orig (Erw = Eri = 1)
  }
  R Psacw = qc * C.K_sacw * MOMs_2ds * fr;
  R Pgacw = qc * C.K_gacw * RLMDg_3dg * fr;
  R Praci = qi * C.K_raci * RLMDr_3dr * fr;
  R Psaci = qi * C.K_saci * Esi_mod * MOMs_2ds * fr;
  R Piacr = qi * C.K_iacr * RLMDr_6dr * fr;
  const R dvrs = fabsR(Vtr - Vts);
  R Psacr = C.K_sacr * Rdens * dvrs *
            (C.GAM_1br * RLMDr_1br * MOMs_2 + C.K_2gam2br * RLMDr_2br * MOMs_1 + C.GAM_3br * RLMDr_3br * MOMs_0);
  R Pgacr = C.K_gacr * Rdens * fabsR(Vtg - Vtr) *
            (C.K_g13 * RLMDr_1br * RLMDg_3 + C.K_g22 * RLMDr_2br * RLMDg_2 + C.GAM_3br * RLMDr_3br * RLMDg);
  R Pracs = C.K_racs * Rdens * dvrs * (R(2.0) * MOMs_0bs * RLMDr_3 + R(2.0) * MOMs_1bs * RLMDr_2 + MOMs_2bs * RLMDr);
  R Pgaci = Z, Pgacs = Z;   // Egi = Egs = 0 unless OPT
  if constexpr (OPT) {
    Pgaci = qi * C.K_gaci * RLMDg_3dg * fr;
    R Egs_mod = C.Egs;
    if (!(warm && C.Egs >= Z)) Egs_mod = dmin(C.Egs, C.Egs * mth.exp(C.gamma_gacs * temc));
    Pgacs = C.K_gacs * Rdens * Egs_mod * fabsR(Vtg - Vts) *
            (R(2.0) * MOMs_0bs * RLMDg_3 + R(2.0) * MOMs_1bs * RLMDg_2 + MOMs_2bs * RLMDg);
  }

  // autoconversion, :1147-1172 (KK2000; only the second Praut_kk assignment is live)
  const R rhoqc = densR * qc * R(1000.0);
  R Praut = Z;   // K_aut * pow(0, 2.47) = 0
  if (kk) {
    R K_aut = C.K_aut;
    if constexpr (OPT) {
      if (C.opt_indir != Z) K_aut = C.kk_aut * mth.pow(Nc, R(-1.79));
    }
    if (gt_z(qc)) Praut = K_aut * mth.pow(qc, R(2.47));
  } else {
    // Berry (1968), :1145-1147
    R Dc = C.Dc_berry;
    if constexpr (OPT) {
      if (C.opt_indir != Z) Dc = R(0.146) - R(5.964E-2) * mth.log(Nc / R(2000.0));
    }
    Praut = Rdens * R(1.67E-5) * rhoqc * rhoqc / (R(5.0) + R(3.66E-2) * Nc / (Dc * rhoqc + R(EPS)));
  }
  R Psaut = rate_on(betai * (qi - C.qicrt_saut));

  // evaporation, sublimation, melting and freezing, :1174-1247
  const R Ka = (R(2.428E-2) + R(7.47E-5) * temc);
  const R KdD = (R(2.222E-5) + R(1.37E-7) * temc) * R(PSTD) / pre * densR;   // Kd * dens
  const R rNu = densR / (R(1.718E-5) + R(5.28E-8) * temc);                 // 1 / Nu
  const R rKaT = ONE / (Ka * tempR);
  const R xi = KdD * qsati;
  const R Giv = xi / (R(LHS0) * rKaT * (C.LovR_ice * rtem - ONE) * xi + ONE);
  const R Gil = Ka * temc * C.rLHF0;
  R Prevp = Z;
  if (rain) {
    const R xl = KdD * qsatl;
    const R Glv = xl / (R(LHV0) * rKaT * (C.LovR_liq * rtem - ONE) * xl + ONE);
    const R ventr = C.K_ventr1 * RLMDr_2 + C.K_ventr2 * sqrtR(C.Cr * fr * rNu * RLMDr_5dr);
    Prevp = C.K_revp * Rdens * (ONE - minc(Sliq, ONE)) * Glv * ventr;
  }
  const R rhoqi = maxc(densR * qi, R(EPS));
  // with no ice, rhoqi = EPS and XNi, Di take the constant values folded on the host
  R XNi = C.XNi_eps, Di = C.Di_eps;
  if (gt_c(rhoqi, R(EPS))) {
    XNi = minc(maxc(R(5.38E+7) * mth.pow(rhoqi, R(0.75)), R(1.0E+3)), R(1.0E+6));
    const R XMi = rhoqi / XNi;
    Di = minc(C.Di_a * sqrtR(XMi), C.Di_max);
  }
  R tmp = R(4.0) * Di * XNi * Rdens * (Sice - ONE) * Giv;
  R Pidep = sel(sps, tmp);
  R Pisub = sel(!sps, -tmp);
  const bool below40 = lt_z(temc + R(40.0));
  R Pihom = below40 ? dqc_dt : Z;
  const R efrz = mth.exp(-C.A_frz * temc) - ONE;
  R Pihtr = (!below40 && !warm) ? densR * (qc * qc) * C.K_ihtr * efrz : Z;
  R Pimlt = warm ? dqi_dt : Z;
  // ventilation of snow and graupel: without the species their moments /
  // slope terms are exact zeros and so is the sum (+0, skipped with its root)
  const R vents = (is_zero(MOMs_1) && is_zero(MOMs_5ds_h)) ? Z : R(0.65) * MOMs_1 + C.K_vents2 * sqrtR(fr * rNu) * MOMs_5ds_h;
  tmp = C.K_2pi * Rdens * (Sice - ONE) * Giv * vents;
  R Psdep = sel(sps, tmp);
  R Pssub = sel(!sps, -tmp);
  R Psmlt = maxz(C.K_2pi * Rdens * Gil * vents + C.K_clf * temc * (Psacw + Psacr));
  const R ventg = (is_zero(RLMDg_2) && is_zero(RLMDg_5dg)) ? Z
                                                  : C.K_ventg1 * RLMDg_2 + C.K_ventg2 * sqrtR(C.Cg * fr * rNu * RLMDg_5dg);
  tmp = C.K_gdep * Rdens * (Sice - ONE) * Giv * ventg;
  R Pgdep = sel(sps, tmp);
  R Pgsub = sel(!sps, -tmp);
  R Pgmlt = maxz(C.K_gdep * Rdens * Gil * ventg + C.K_clf * temc * (Pgacw + Pgacr));
  R Pgfrz = C.K_gfrz * Rdens * efrz * RLMDr_7;

  // Bergeron process (:1239-1247) with Bergeron_param (:1834-1890); it
  // contributes only when sw_bergeron = 1 (-30 <= temc <= 0, sw_expice = 0)
  // and iceflg = 1 (temc < 0)
  const bool expice = !OPT || C.opt_expice != Z;
  const bool cold = !warm;   // iceflg == 1
  R Psfw = Z, Psfi = Z;
  if constexpr (OPT) {
    if (!expice && cold && !(temc + R(30.0) < Z)) {
      const R tb = dmin(dmax(temc, R(-30.99)), Z);
      const int it = int(-val_of(tb));   // the table row: piecewise constant in tb
      const R fact = -(tb + R(it - 1));
      const R a2 = (ONE - fact) * C.berg_a2[it] + fact * C.berg_a2[it + 1];
      const R ma2 = ONE - a2;
      const R a1 = ((ONE - fact) * C.berg_a1[it] + fact * C.berg_a1[it + 1]) * mth.pow(R(1.0E-3), ma2);
      const R dt1 = (mth.exp(C.log_mi50 * ma2) - mth.exp(C.log_mi40 * ma2)) / (a1 * ma2);
      const R Ni50 = qi * dtR / (C.mi50 * dt1);
      Psfw = Ni50 * (a1 * mth.pow(C.mi50, a2) + C.K_berg_w * densR * qc);
      Psfi = qi / dt1;
    }
  }

  // limiters, :1249-1296 (iceflg selects; sw_expice = 1 unless OPT; Pgaut = 0)
  Pigen = sel(cold && expice, min_nn(Pigen, dqv_dt));
  Pidep = sel(cold && expice, min_nn(Pidep, dqv_dt));
  Psdep = sel(cold, min_nn(Psdep, dqv_dt));
  Pgdep = sel(cold, min_nn(Pgdep, dqv_dt));
  Pracw = Pracw + sel(warm, Psacw) + sel(warm, Pgacw);
  Praut = min_nn(Praut, dqc_dt);
  Pracw = min_nn(Pracw, dqc_dt);
  Pihom = sel(cold && expice, min_nn(Pihom, dqc_dt));
  Pihtr = sel(cold && expice, min_nn(Pihtr, dqc_dt));
  Psacw = sel(cold, min_nn(Psacw, dqc_dt));
  if constexpr (OPT) Psfw = sel(cold, min_nn(Psfw, dqc_dt));
  Pgacw = sel(cold, min_nn(Pgacw, dqc_dt));
  Prevp = min_nn(Prevp, dqr_dt);
  Piacr = sel(cold, min_nn(Piacr, dqr_dt));
  Psacr = sel(cold, min_nn(Psacr, dqr_dt));
  Pgacr = sel(cold, min_nn(Pgacr, dqr_dt));
  Pgfrz = sel(cold, min_nn(Pgfrz, dqr_dt));
  Pisub = sel(cold && expice, min_nn(Pisub, dqi_dt));
  Pimlt = sel(warm && expice, min_nn(Pimlt, dqi_dt));
  Psaut = sel(cold, min_nn(Psaut, dqi_dt));
  Praci = sel(cold, min_nn(Praci, dqi_dt));
  Psaci = sel(cold, min_nn(Psaci, dqi_dt));
  if constexpr (OPT) {
    Psfi = sel(cold, min_nn(Psfi, dqi_dt));
    Pgaci = sel(cold, min_nn(Pgaci, dqi_dt));
  }
  Pssub = sel(cold, min_nn(Pssub, dqs_dt));
  Psmlt = sel(warm, min_nn(Psmlt, dqs_dt));
  Pracs = sel(cold, min_nn(Pracs, dqs_dt));
  if constexpr (OPT) Pgacs = min_nn(Pgacs, dqs_dt);
  Pgsub = sel(cold, min_nn(Pgsub, dqg_dt));
  Pgmlt = sel(warm, min_nn(Pgmlt, dqg_dt));
  R Piacr_s = sel(!d1, Piacr);
  R Piacr_g = sel(d1, Piacr);
  R Praci_s = sel(!d1, Praci);
  R Praci_g = sel(d1, Praci);
  R Psacr_s = sel(d2, Psacr);
  R Psacr_g = sel(!d2, Psacr);
  Pracs = sel(!d2, Pracs);

  // loss limiters, :1298-1477: fac = 1 when production >= loss - EPS,
  // else min(-dq/dt / net, 1) (the reference's (net - fac_sw) is net there)
  auto limiter = [&](R net, R dq) {
    return is_nonneg(net + R(EPS)) ? ONE : dmin(-dq / net, ONE);
  };
  // Scaling by fac = 1 is exact and skipped.  The tendencies below are the
  // nets the limiters form (same terms, same order) where no later scaling
  // changed their rates.  lc .. lg: the QC, QI, QR, QV, QS, QG limiter scaled
  // its rates.
  bool lc, li, lr, lv, ls, lg;
  R fac, net_c, net_i, net_r, net_s, net_g;
  if constexpr (!OPT) {
    net_c = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw;  // [QC]
    fac = limiter(net_c, dqc_dt);
    lc = !is_one(fac);
    if (lc) {
      Pimlt *= fac; Praut *= fac; Pracw *= fac; Pihom *= fac; Pihtr *= fac; Psacw *= fac; Pgacw *= fac;
    }
    net_i = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g;  // [QI]
    fac = limiter(net_i, dqi_dt);
    li = !is_one(fac);
    if (li) {
      Pigen *= fac; Pidep *= fac; Pihom *= fac; Pihtr *= fac; Pisub *= fac; Pimlt *= fac; Psaut *= fac;
      Praci_s *= fac; Psaci *= fac; Praci_g *= fac;
    }
  } else {
    net_c = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Psfw - Pgacw;  // [QC]
    fac = limiter(net_c, dqc_dt);
    lc = !is_one(fac);
    if (lc) {
      Pimlt *= fac; Praut *= fac; Pracw *= fac; Pihom *= fac; Pihtr *= fac; Psacw *= fac; Psfw *= fac; Pgacw *= fac;
    }
    net_i = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Psfi - Praci_g - Pgaci;  // [QI]
    fac = limiter(net_i, dqi_dt);
    li = !is_one(fac);
    if (li) {
      Pigen *= fac; Pidep *= fac; Pihom *= fac; Pihtr *= fac; Pisub *= fac; Pimlt *= fac; Psaut *= fac;
      Praci_s *= fac; Psaci *= fac; Psfi *= fac; Praci_g *= fac; Pgaci *= fac;
    }
  }
  net_r = +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz;  // [QR]
  fac = limiter(net_r, dqr_dt);
  lr = !is_one(fac);
  if (lr) {
    Praut *= fac; Pracw *= fac; Psmlt *= fac; Pgmlt *= fac; Prevp *= fac; Piacr_s *= fac; Psacr_s *= fac;
    Piacr_g *= fac; Psacr_g *= fac; Pgacr *= fac; Pgfrz *= fac;
  }
  fac = limiter(+Prevp + Pisub + Pssub + Pgsub - Pigen - Pidep - Psdep - Pgdep, dqv_dt);  // [QV]
  lv = !is_one(fac);
  if (lv) {
    Prevp *= fac; Pisub *= fac; Pssub *= fac; Pgsub *= fac; Pigen *= fac; Pidep *= fac; Psdep *= fac; Pgdep *= fac;
  }
  if constexpr (!OPT) {
    net_s = +Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs;  // [QS]
    fac = limiter(net_s, dqs_dt);
    ls = !is_one(fac);
    if (ls) {
      Psdep *= fac; Psacw *= fac; Piacr_s *= fac; Psacr_s *= fac; Psaut *= fac; Praci_s *= fac; Psaci *= fac;
      Pssub *= fac; Psmlt *= fac; Pracs *= fac;
    }
    net_g = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt;  // [QG]
    fac = limiter(net_g, dqg_dt);
    lg = !is_one(fac);
    if (lg) {
      Pgdep *= fac; Pgacw *= fac; Piacr_g *= fac; Psacr_g *= fac; Pgacr *= fac; Pgfrz *= fac; Praci_g *= fac;
      Pracs *= fac; Pgsub *= fac; Pgmlt *= fac;
    }
  } else {
    net_s = +Psdep + Psacw + Psfw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci + Psfi - Pssub - Psmlt - Pracs - Pgacs;
    fac = limiter(net_s, dqs_dt);  // [QS]
    ls = !is_one(fac);
    if (ls) {
      Psdep *= fac; Psacw *= fac; Psfw *= fac; Piacr_s *= fac; Psacr_s *= fac; Psaut *= fac; Praci_s *= fac;
      Psaci *= fac; Psfi *= fac; Pssub *= fac; Psmlt *= fac; Pracs *= fac; Pgacs *= fac;
    }
    net_g = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pgaci + Pracs + Pgacs - Pgsub - Pgmlt;
    fac = limiter(net_g, dqg_dt);  // [QG]
    lg = !is_one(fac);
    if (lg) {
      Pgdep *= fac; Pgacw *= fac; Piacr_g *= fac; Psacr_g *= fac; Pgacr *= fac; Pgfrz *= fac; Praci_g *= fac;
      Pgaci *= fac; Pracs *= fac; Pgacs *= fac; Pgsub *= fac; Pgmlt *= fac;
    }
  }

  // tendencies, :1479-1559.  A species' net above stands unless a limiter at
  // or after it scaled one of its rates: QC's by QC, QI, QR, QS, QG; QI's by
  // QI, QV, QS, QG; QR's by QR, QV, QS, QG; QS's by QS, QG; QG's by QG.
  R qc_t = net_c, qr_t = net_r, qi_t = net_i, qs_t = net_s, qg_t = net_g;
  if (lr | lv | ls | lg) qr_t = +Praut + Pracw + Psmlt + Pgmlt - Prevp - Piacr_s - Psacr_s - Piacr_g - Psacr_g - Pgacr - Pgfrz;
  if constexpr (!OPT) {
    if (lc | li | lr | ls | lg) qc_t = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Pgacw;
    if (li | lv | ls | lg) qi_t = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Praci_g;
    if (ls | lg) qs_t = +Psdep + Psacw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci - Pssub - Psmlt - Pracs;
    if (lg) qg_t = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pracs - Pgsub - Pgmlt;
  } else {
    if (lc | li | lr | ls | lg) qc_t = +Pimlt - Praut - Pracw - Pihom - Pihtr - Psacw - Psfw - Pgacw;
    if (li | lv | ls | lg)
      qi_t = +Pigen + Pidep + Pihom + Pihtr - Pisub - Pimlt - Psaut - Praci_s - Psaci - Psfi - Praci_g - Pgaci;
    if (ls | lg)
      qs_t = +Psdep + Psacw + Psfw + Piacr_s + Psacr_s + Psaut + Praci_s + Psaci + Psfi - Pssub - Psmlt - Pracs - Pgacs;
    if (lg) qg_t = +Pgdep + Pgacw + Piacr_g + Psacr_g + Pgacr + Pgfrz + Praci_g + Pgaci + Pracs + Pgacs - Pgsub - Pgmlt;
  }
  qc_t = max_nd(qc_t, dqc_dt);
  qr_t = max_nd(qr_t, dqr_dt);
  qi_t = max_nd(qi_t, dqi_dt);
  qs_t = max_nd(qs_t, dqs_dt);
  qg_t = max_nd(qg_t, dqg_dt);
  const R qv_t = -(qc_t + qr_t + qi_t + qs_t + qg_t);
  D drq[6];
  if constexpr (kMixed) {
    // The tracer changes rhog q_t dt of the FP32 rates, formed in FP32 and
    // added to the FP64 budgets.  A species whose loss reached its whole
    // content leaves exactly nothing (the FP64 path leaves a rounding residue
    // of the same size as the reference's; FP32 rates would leave one 10^9
    // times larger), and the vapour takes the balance so that total water
    // stays exact.
    const R rgdt = R(rhog * dt);
    const R qt[6] = {qv_t, qc_t, qr_t, qi_t, qs_t, qg_t};
    const R lim[6] = {dqv_dt, dqc_dt, dqr_dt, dqi_dt, dqs_dt, dqg_dt};
    D sum = D(0.0);
#pragma unroll
    for (int n = 1; n <= 5; ++n) {
      drq[n] = (qt[n] <= -lim[n] && lim[n] > Z) ? -rq[n] : D(qt[n] * rgdt);
      sum += drq[n];
    }
    drq[0] = -sum;
  } else {
    drq[0] = rhog * D(qv_t) * dt;
    drq[1] = rhog * D(qc_t) * dt;
    drq[2] = rhog * D(qr_t) * dt;
    drq[3] = rhog * D(qi_t) * dt;
    drq[4] = rhog * D(qs_t) * dt;
    drq[5] = rhog * D(qg_t) * dt;
  }
  o.Vtr = D(Vtr);
  o.Vts = D(Vts);
  o.Vtg = D(Vtg);
  o.Vti = D(Vti);

  // effective radius and cloud top, :1566-1592
  {
    const R r2_min = R(1.0E-10), q_min = R(1.0E-5);
    R K_xf = C.K_xf, K_r2c = C.K_r2c;
    if constexpr (OPT) {
      if (C.opt_indir != Z) {
        K_xf = R(1.0E-9) / Nc;
        K_r2c = C.coef_dgam * (Nc * R(1.0E+6));
      }
    }
    const R rf_qc = mth.pow(C.coef_xf * (rhoqc * K_xf) + R(EPS), R(0.33333333));
    const R r2_qc = K_r2c * (rf_qc * rf_qc);
    const R r2_qr = C.K_r2r * RLMDr_3;
    const R r3_qc = C.coef_xf * densR * qc;
    const R r3_qr = C.coef_xf * densR * qr;
    const R r2 = r2_qc + r2_qr;
    const bool big = ge_c(r2, r2_min);
    const R rceff = big ? (r3_qc + r3_qr) / r2 : Z;
    const bool top = !big && ge_c(qc + qr, q_min);
    o.rceff = D(rceff);
    o.rctop = top ? D(rceff) : D(UNDEF);
    o.tctop = top ? temp : D(UNDEF);
    o.rceff_cld = ge_c(r2_qc, r2_min) ? D(r3_qc / r2_qc) : D(0.0);
  }

  // ---- TagUpdateRHOGQ / RHOGE / MassConc / TEM, mod_mp_nsw6.cpp:692-744
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] += drq[n];
  rhoge = rhoge - LHV0 * drq[I_QV] + LHF0 * drq[I_QI] + LHF0 * drq[I_QS] + LHF0 * drq[I_QG];
  o.q[0] = qn[0];
  if constexpr (kMixed) {
    // q from the shared reciprocal, T = rhoge / (rhog CVdry) (cv = CVdry as above)
#pragma unroll
    for (int n = 1; n <= 5; ++n) o.q[n] = rq[n] * rrhog;
    o.tem = rhoge * rrhog * (1.0 / CVDRY);
  } else {
#pragma unroll
    for (int n = 1; n <= 5; ++n) o.q[n] = div_rn(rq[n], rhog, rrhog);
    D qd2 = D(1.0);
#pragma unroll
    for (int n = 1; n <= 5; ++n) qd2 = qd2 - o.q[n];
    D cva = qd2 * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cva = cva + o.q[n] * CVDRY;
    o.tem = rhoge / (rhog * cva);
  }
  o.rhog = rhog;
  o.rhoge = rhoge;
#pragma unroll
  for (int n = 0; n < 6; ++n) o.rhogq[n] = rq[n];
}

// Half-level velocity wh(j) of vadv1d_prep (mod_vadv1d.cpp:270-282) for a column
// accessor wp(j).
template <class R, class WP>
__device__ __forceinline__ R vadv_wh(const WP& wp, int j, int mkmin, int mkmax) {
  if (j >= mkmin + 1 && j <= mkmax) return R(0.5) * (wp(j - 1) + wp(j));
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
// The same from the half-level velocities wh(j) themselves (an accessor).
template <class R, class G, class WH>
__device__ __forceinline__ R vadv_zdis_wh(const WH& wh, const G* rdz, const G* rdzs, int k, int mkmin, R dt, R hdt2,
                                          R sdt3) {
  if (k == mkmin) {
    const R w0 = wh(mkmin), wpp = wh(mkmin + 1);
    return fmaR(-hdt2 * w0, (wpp - w0) * rdz[mkmin], dt * w0);
  }
  const R wm = wh(k - 1);
  const R w0 = wh(k);
  const R wpp = wh(k + 1);
  const R r = (wpp - wm) * rdzs[k];
  const R c = R(2.0) * rdzs[k] * fmaR(wpp - w0, rdz[k], -(w0 - wm) * rdz[k - 1]);
  const R t3 = sdt3 * w0 * fmaR(w0, c, r * r);
  return fmaR(-hdt2 * w0, r, fmaR(dt, w0, t3));
}

template <class R, class G, class WP>
__device__ __forceinline__ R vadv_zdis(const WP& wp, const G* rdz, const G* rdzs, int k, int mkmin, int mkmax, R dt,
                                       R hdt2, R sdt3) {
  auto wh = [&](int j) { return vadv_wh<R>(wp, j, mkmin, mkmax); };
  return vadv_zdis_wh<R>(wh, rdz, rdzs, k, mkmin, dt, hdt2, sdt3);
}

}  // namespace nsw6
