// One whole NSW6 step of one column, written as a template over the scalar
// type T, for the tangent-linear (T = Dual) and adjoint (T = RVar) kernels and
// for their check against the production kernels (T = double).
//
// It performs, serially over the levels of one column, exactly the operations
// of nsw6_cell_kernel followed by nsw6_column_kernel in the same order, so that
// the T = double instance reproduces the FP64 step bit for bit:
//   nsw6_cell per interior cell (mod_mp_nsw6.cpp:439-744), the departure
//   distances of vadv1d_prep (mod_vadv1d.cpp:231-391), the transport of QR,
//   QS, QG with the flux integrals of vadv1d_getflux_new (mod_vadv1d.cpp:
//   393-450, mod_precip_transport.cpp:767-955), the tendencies and KIN2EIN
//   (:956-1011), the final thermodynamics, the saturation adjustment
//   (mod_satadjust.cpp:274-362, 771-896) and the closing negative filter.
//
// Not differentiated (the scheme's discrete choices): the departure cells and
// the region-wide bounds of the flux integrals (kcell_min / kcell_max, taken
// from the FP64 step of the same state), the small-flux filter |F| < EPS, and
// every limiter and switch, whose derivative is that of the branch taken.  The
// saturation adjustment is differentiated implicitly at its converged
// temperature: with F(T) = T cv(T) + qsat(T) LHV0 - Emoist = 0,
// dT = -dF|_T / (dF/dT).
#pragma once

#include "nsw6_ad.cuh"
#include "nsw6_cell.cuh"
#include "nsw6_common.cuh"

namespace nsw6 {

constexpr int KA = 48;   // largest kall of the derivative kernels

template <class T>
struct ColState {
  // read and written
  T rhog[KA], rhoge[KA], rhogvx[KA], rhogvy[KA], rhogvz[KA], rhogw[KA];
  T rhogq[6][KA], tem[KA], q[6][KA];
  // read only
  T vx[KA], vy[KA], vz[KA], gsgam2[KA], gsgam2h[KA], gam2[KA], gam2h[KA], z[KA];
  T ix, iy, iz, jx, jy, jz;
  // written only
  T rho[KA], pre[KA], qd[KA], re_liquid[KA], re_cld[KA], GPREC[KA];
  T precip0, precip1, lh_heat, p_rhoe, p_rhophi, p_rhokin, rctop, rwtop, tctop;
};

template <class T>
struct ColWork {
  T vt[3][KA], zdis[6][KA];
  T rgs[KA], vi[KA], vj[KA], kinh[KA], kinv[KA];
  T drhoe[KA], drhophi[KA], dkinh[KA], dkinv[KA], drhogu[KA], drhogv[KA], drhogw[KA], dq[3][KA];
  T base[KA], rhof[KA], f[KA];
  unsigned char kc[KA];
};

// The parameter-dependent scheme constants as functions of the parameters p
// (beta_saut, qicrt_saut, Cr, Cs, Cg, ice_nuc, kk_aut); values as built on the
// host, derivatives of the factors folded from them (make_consts).
template <class T>
__device__ __forceinline__ void consts_with_params(const Consts& c, const T* p, ConstsT<T>& r) {
  const double* src = reinterpret_cast<const double*>(&c);
  T* dst = reinterpret_cast<T*>(&r);
  for (size_t i = 0; i < sizeof(Consts) / sizeof(double); ++i) dst[i] = T(src[i]);
  r.beta_saut = p[0];
  r.qicrt_saut = p[1];
  r.Cr = p[2];
  r.Cs = p[3];
  r.Cg = p[4];
  r.ice_nuc = p[5];
  r.kk_aut = p[6];
  r.K_vtr = dep(c.K_vtr, p[2], c.K_vtr / c.Cr);
  r.K_raci = dep(c.K_raci, p[2], c.K_raci / c.Cr);
  r.K_iacr = dep(c.K_iacr, p[2], c.K_iacr / c.Cr);
  r.K_vts = dep(c.K_vts, p[3], c.K_vts / c.Cs);
  r.K_sacw = dep(c.K_sacw, p[3], c.K_sacw / c.Cs);
  r.K_saci = dep(c.K_saci, p[3], c.K_saci / c.Cs);
  r.K_vents2 = dep(c.K_vents2, p[3], 0.5 * c.K_vents2 / c.Cs);
  r.K_vtg = dep(c.K_vtg, p[4], c.K_vtg / c.Cg);
  r.K_gacw = dep(c.K_gacw, p[4], c.K_gacw / c.Cg);
  r.K_aut = dep(c.K_aut, p[6], c.K_aut / c.kk_aut);
}
__device__ __forceinline__ void consts_with_params(const Consts& c, const double*, Consts& r) { r = c; }

template <class T>
__device__ __forceinline__ T flux_integral_t(const T* rhof, const double* dz, int k, int kc, const T& zdis0, int bmn,
                                             int bmx) {
  T f = T(0.0), zdis = zdis0;
  if (!(bmn == k && bmx == k)) {
    for (int k2 = bmn; k2 <= bmx; ++k2) f = fmaR(rhof[k2], T(k2 > kc ? dz[k2] : (k2 < kc ? -dz[k2] : 0.0)), f);
    if (bmx != kc) zdis = zdis0 - T(bmx > kc ? dz[bmx] : -dz[bmx]);
  }
  f = fmaR(rhof[kc], zdis, f);
  return fabsR(f) >= T(EPS) ? f : T(0.0);
}

// Column bounds of the flux integrals from the region extrema keys, as the
// column kernel forms them (mod_vadv1d.cpp:316-353).
__device__ __forceinline__ void column_bounds(const double* gzh, const double* gzs, int K, int kmin, int kmax,
                                              const unsigned long long* zmax, const unsigned long long* zmin,
                                              int (*bmn)[KA], int (*bmx)[KA]) {
  for (int s = 0; s < 6; ++s)
    for (int k = 0; k < K; ++k) {
      const int half = s / 3;
      const int mkmin = half ? kmin + 1 : kmin;
      const double* zh = half ? gzs : gzh;
      int lo = k, hi = k;
      if (k >= mkmin && k <= kmax) {
        const unsigned long long kx = zmax[s * K + k], kn = zmin[s * K + k];
        double zzmax = DBL_MIN, zzmin = DBL_MIN;
        if (kx != 0ull) {
          const double v = key_value(kx);
          zzmax = v > zzmax ? v : zzmax;
        }
        if (kn != ~0ull) {
          const double v = key_value(kn);
          zzmin = v < zzmin ? v : zzmin;
        }
        if (zzmax > 0.0) {
          for (int k2 = k; k2 >= mkmin; --k2)
            if ((zh[k2] <= zh[k] - zzmax) && (zh[k2 + 1] > zh[k] - zzmax)) {
              lo = k2;
              break;
            }
        }
        if (zzmin < 0.0) {
          for (int k2 = k; k2 <= kmax; ++k2)
            if ((zh[k2] <= zh[k] - zzmin) && (zh[k2 + 1] > zh[k] - zzmin)) {
              hi = k2;
              break;
            }
        }
      }
      bmn[s][k] = lo;
      bmx[s][k] = hi;
    }
}

// Departure cell (mod_vadv1d.cpp:355-389), as in the column kernel.
__device__ __forceinline__ int departure_cell_t(const double* zh, int k, double zdis, int bmn, int bmx, int mkmin,
                                                int mkmax) {
  int kc;
  if (bmn == k && bmx == k) {
    kc = k;
  } else {
    kc = 0;
    const double dep = zh[k] - zdis;
    for (int k2 = bmn; k2 <= bmx; ++k2) {
      const bool s1 = dep >= zh[k2];
      const bool s2 = zh[k2 + 1] >= dep;
      const int tmp = (s1 == s2) ? k2 : -k2;
      kc = kc > tmp ? kc : tmp;
    }
  }
  if (kc == 0) kc = mkmin;
  if (kc == mkmax + 1) kc = mkmax;
  return kc;
}

// Saturation-adjustment temperature of one cell.  The Newton iteration runs on
// the values exactly as in the column kernel; its result enters T through the
// implicit-function derivative at the converged point.  Returns 0, or the
// error code (3 no convergence, 4 non-finite) with *iters set.
template <class T>
__device__ __forceinline__ int satadjust_t(const Consts& C, const FastMath& fm, int itelim, const T& ein_moist,
                                           const T& qsum, const T& rho_l, T* q, T& tem, int* iters) {
  // qd_l = 1 - sum(q[1..5]) with q[QC] = 0 at entry
  T qd_l = T(1.0);
#pragma unroll
  for (int n = 1; n <= 5; ++n) qd_l = qd_l - q[n];
  double tv = val(tem);
  const double qsumv = val(qsum), rhov = val(rho_l), emv = val(ein_moist), qdv = val(qd_l);
  double qv[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) qv[n] = val(q[n]);
  double rtem = 1.0 / (dmax(tv, TEM_MIN));
  double psat = PSAT0 * fm.exp(C.LovR_liq * (C.RTEM00 - rtem));
  double qsat = psat / (rhov * RVAP * tv);
  if (!(qsumv - qsat > EPS)) return 0;
  bool converged = false;
  int ite;
  double tprev = tv;
  for (ite = 0; ite < itelim; ++ite) {
    tprev = tv;
    rtem = 1.0 / (dmax(tv, TEM_MIN));
    psat = PSAT0 * fm.exp(C.LovR_liq * (C.RTEM00 - rtem));
    qsat = psat / (rhov * RVAP * tv);
    qv[I_QV] = qsat;
    qv[I_QC] = qsumv - qsat;
    double cv = qdv * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cv = cv + qv[n] * CVDRY;
    const double emoist_new = tv * cv + qv[I_QV] * LHV0;
    const double dqsat_dT = C.LovR_liq * rtem * rtem * qsat;
    const double demoist_dT = cv + dqsat_dT * LHV0;
    const double dtemp = (emoist_new - emv) / demoist_dT;
    tv = tv - dtemp;
    if (fabs(dtemp) < C.dtemp_criteria) {
      converged = true;
      break;
    }
    if (tv * 0.0 != 0.0) break;
  }
  *iters = ite;
  if (!converged) {
    tem = T(tv);
    q[I_QV] = T(qv[I_QV]);
    q[I_QC] = T(qv[I_QC]);
    return (tv * 0.0 != 0.0) ? 4 : 3;
  }
  // F(T) = T cv(T) + qsat(T) LHV0 - Emoist with cv = (qd_l + qsum - qsat +
  // sum q[2..5]) CVdry, evaluated with T-typed inputs at the converged value
  const double ts = tprev;
  const T Tc = T(ts);
  const T qsT = T(PSAT0) * T(fm.exp(C.LovR_liq * (C.RTEM00 - 1.0 / dmax(ts, TEM_MIN)))) / (rho_l * RVAP * Tc);
  T cvT = qd_l * CVDRY + (qsum - qsT) * CVDRY;
#pragma unroll
  for (int n = 2; n <= 5; ++n) cvT = cvT + q[n] * CVDRY;
  const T F = Tc * cvT + qsT * LHV0 - ein_moist;
  const double rts = 1.0 / ts;
  const double qs_v = val(qsT);
  const double dqs = qs_v * (C.LovR_liq * rts * rts - rts);   // d qsat / dT (T > TEM_MIN)
  const double cv_v = val(cvT);
  const double FT = cv_v - ts * dqs * CVDRY + dqs * LHV0;
  const T temI = T(ts) - (F - T(val(F))) * (1.0 / FT);
  // q[QV] = qsat(T), q[QC] = qsum - qsat(T) with the derivative of T through temI
  const T qsI = qsT + (temI - Tc) * dqs;
  q[I_QV] = with_value(qsI, qv[I_QV]);
  q[I_QC] = with_value(qsum - qsI, qv[I_QC]);
  tem = with_value(temI, tv);
  return 0;
}

// The mixed-phase saturation adjustment (satadjust_all, mod_satadjust.cpp:
// 620-769, with the scheme switch explicit_icegen = 0) of one cell, as the
// column kernel iterates it: liquid and ice saturation blended by alpha(T)
// between sat_llimit and sat_ulimit, the excess split into cloud water and
// cloud ice by alpha.  q[QC] and q[QI] are 0 at entry, qsum = qv + qc + qi
// and ein_moist carries -qi LHF0.  The derivative is the implicit one at the
// last iterate ts: F(T) = T cv + qsat LHV0 - qi LHF0 - Emoist, with the
// outputs linear in T about ts.  Its T-slopes are the exact ones (d qsat / dT
// = qsat (LovR / T^2 - 1 / T), cv = qd_l + qc + q2 + qi + q4 + q5 in CVdry),
// not the iteration's approximate ones.
template <class T>
__device__ __forceinline__ int satadjust_all_t(const Consts& C, const FastMath& fm, int itelim, const T& ein_moist,
                                               const T& qsum, const T& rho_l, T* q, T& tem, int* iters) {
  T qd_l = T(1.0);
#pragma unroll
  for (int n = 1; n <= 5; ++n) qd_l = qd_l - q[n];
  const double UL = C.sat_ulimit, LL = C.sat_llimit;
  double tv = val(tem);
  const double qsumv = val(qsum), rhov = val(rho_l), emv = val(ein_moist), qdv = val(qd_l);
  double qv[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) qv[n] = val(q[n]);
  {
    const double rtem = 1.0 / (dmax(tv, TEM_MIN));
    double psat = PSAT0 * fm.exp(C.LovR_liq * (C.RTEM00 - rtem));
    const double alpha = dmin(dmax((tv - LL) / (UL - LL), 0.0), 1.0);
    const double psati = PSAT0 * fm.exp(C.LovR_ice * (C.RTEM00 - rtem));
    psat = psat * alpha + psati * (1.0 - alpha);
    const double qsat = psat / (rhov * RVAP * tv);
    if (!(qsumv - qsat > EPS)) return 0;
  }
  bool converged = false;
  int ite;
  double tprev = tv, alpha_s = 0.0, dalpha_s = 0.0, psatl_s = 0.0, psati_s = 0.0;
  for (ite = 0; ite < itelim; ++ite) {
    tprev = tv;
    const double alpha = dmin(dmax((tv - LL) / (UL - LL), 0.0), 1.0);
    const double rtem = 1.0 / (dmax(tv, TEM_MIN));
    const double psatl = PSAT0 * fm.exp(C.LovR_liq * (C.RTEM00 - rtem));
    const double psati = PSAT0 * fm.exp(C.LovR_ice * (C.RTEM00 - rtem));
    const double psat = psatl * alpha + psati * (1.0 - alpha);
    const double qsatl = psatl / (rhov * RVAP * tv);
    const double qsati = psati / (rhov * RVAP * tv);
    const double qsat = psat / (rhov * RVAP * tv);
    qv[I_QV] = qsat;
    qv[I_QC] = (qsumv - qsat) * alpha;
    qv[I_QI] = (qsumv - qsat) * (1.0 - alpha);
    double cv = qdv * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cv = cv + qv[n] * CVDRY;
    const double emoist_new = tv * cv + qv[I_QV] * LHV0 - qv[I_QI] * LHF0;
    const double dalpha_dT = (!(UL - tv < 0.0) && !(tv - LL < 0.0)) ? 1.0 / (UL - LL) : 0.0;
    const double t2 = tv * tv;
    const double dqsatl_dT = (C.LovR_liq / t2) * qsatl;
    const double dqsati_dT = (C.LovR_ice / t2) * qsati;
    const double dqsat_dT = qsatl * dalpha_dT + dqsatl_dT * alpha - qsati * dalpha_dT + dqsati_dT * (1.0 - alpha);
    const double dqc_dT = (qsumv - qsat) * dalpha_dT - dqsat_dT * alpha;
    const double dqi_dT = -(qsumv - qsat) * dalpha_dT - dqsat_dT * (1.0 - alpha);
    const double dcv_dT = dqsat_dT * CVDRY + dqc_dT * CVDRY + dqi_dT * CVDRY;
    const double demoist_dT = tv * dcv_dT + cv + dqsat_dT * LHV0 - dqi_dT * LHF0;
    const double dtemp = (emoist_new - emv) / demoist_dT;
    alpha_s = alpha;
    dalpha_s = dalpha_dT;
    psatl_s = psatl;
    psati_s = psati;
    tv = tv - dtemp;
    if (fabs(dtemp) < C.dtemp_criteria) {
      converged = true;
      break;
    }
    if (tv * 0.0 != 0.0) break;
  }
  *iters = ite;
  if (!converged) {
    tem = T(tv);
    q[I_QV] = T(qv[I_QV]);
    q[I_QC] = T(qv[I_QC]);
    q[I_QI] = T(qv[I_QI]);
    return (tv * 0.0 != 0.0) ? 4 : 3;
  }
  // F at the last iterate with the inputs' derivatives (Tc, alpha and the
  // saturation pressures held at their values there)
  const double ts = tprev;
  const T Tc = T(ts);
  const T qsT = T(psatl_s * alpha_s + psati_s * (1.0 - alpha_s)) / (rho_l * RVAP * Tc);
  const T exc = qsum - qsT;
  const T qcT = exc * alpha_s, qiT = exc * (1.0 - alpha_s);
  T cvT = qd_l * CVDRY;
  cvT = cvT + qcT * CVDRY;
  cvT = cvT + q[2] * CVDRY;
  cvT = cvT + qiT * CVDRY;
  cvT = cvT + q[4] * CVDRY;
  cvT = cvT + q[5] * CVDRY;
  const T F = Tc * cvT + qsT * LHV0 - qiT * LHF0 - ein_moist;
  // exact T-slopes at ts
  const double rts = 1.0 / ts;
  const double qsl = psatl_s / (rhov * RVAP * ts), qsi = psati_s / (rhov * RVAP * ts);
  const double dqsl = qsl * (C.LovR_liq * rts * rts - rts), dqsi = qsi * (C.LovR_ice * rts * rts - rts);
  const double qs_v = val(qsT), exc_v = qsumv - qs_v;
  const double dqs = dqsl * alpha_s + dqsi * (1.0 - alpha_s) + (qsl - qsi) * dalpha_s;
  const double dqc = -dqs * alpha_s + exc_v * dalpha_s;
  const double dqi = -dqs * (1.0 - alpha_s) - exc_v * dalpha_s;
  const double FT = val(cvT) + ts * (dqc + dqi) * CVDRY + dqs * LHV0 - dqi * LHF0;
  const T temI = T(ts) - (F - T(val(F))) * (1.0 / FT);
  const T dT = temI - Tc;
  q[I_QV] = with_value(qsT + dT * dqs, qv[I_QV]);
  q[I_QC] = with_value(qcT + dT * dqc, qv[I_QC]);
  q[I_QI] = with_value(qiT + dT * dqi, qv[I_QI]);
  tem = with_value(temI, tv);
  return 0;
}

// The cell phase of one column: nsw6_cell on every interior level (as
// nsw6_cell_kernel), leaving the fall speeds in w.vt.
template <class T, class M>
__device__ void column_cell_phase(const ConstsT<T>& CT, const M& mth, int K, double dt, double rdt,
                                  ColState<T>& s, ColWork<T>& w) {
  const int kmin = 1, kmax = K - 2;
  for (int t = 0; t < 3; ++t)
    for (int k = 0; k < K; ++k) w.vt[t][k] = T(0.0);
  for (int k = kmin; k <= kmax; ++k) {
    CellInT<T> in;
    in.rhog = s.rhog[k];
    in.tem = s.tem[k];
    in.gsgam2 = s.gsgam2[k];
    in.q0 = s.q[0][k];
#pragma unroll
    for (int n = 0; n < 6; ++n) in.rhogq[n] = s.rhogq[n][k];
    CellOutT<T> o;
    nsw6_cell<M, T, T>(CT, mth, dt, rdt, in, o);
    s.rhog[k] = o.rhog;
    s.rhoge[k] = o.rhoge;
    s.tem[k] = o.tem;
#pragma unroll
    for (int n = 0; n < 6; ++n) s.rhogq[n][k] = o.rhogq[n];
#pragma unroll
    for (int n = 1; n < 6; ++n) s.q[n][k] = o.q[n];
    s.re_liquid[k] = o.rceff;
    s.re_cld[k] = o.rceff_cld;
    w.vt[0][k] = o.Vtr;
    w.vt[1][k] = o.Vts;
    w.vt[2][k] = o.Vtg;
    if (k == kmax) {
      s.rctop = o.rctop;
      s.tctop = o.tctop;
      const double sw = (0.5 + copysign(0.5, val(o.tctop) - TEM00));
      s.rwtop = sw * o.rctop + (1.0 - sw) * UNDEF;
    }
  }
}

// The column phase: departure distances from the fall speeds in w.vt,
// transport, KIN2EIN, thermodynamics, saturation adjustment and the closing
// filter (as nsw6_column_kernel).  gr: the grid block [GF_COUNT][K].
template <class T>
__device__ void column_transport_phase(const Consts& C, const FastMath& fm, const double* gr, int K, double dt,
                                       double hdt2, double sdt3, int itelim, const int (*bmn)[KA],
                                       const int (*bmx)[KA], ColState<T>& s, ColWork<T>& w, int* err, int* err_k,
                                       int* err_it);

// The whole step of one column.  mth: exp/log/pow of T.  C: FP64 constants
// (values), CT: the same as T (with the parameter derivatives).  err: first
// error of the column.
template <class T, class M>
__device__ void column_step(const ConstsT<T>& CT, const Consts& C, const M& mth, const FastMath& fm,
                            const double* gr, int K, double dt, double rdt, double hdt2, double sdt3, int itelim,
                            const int (*bmn)[KA], const int (*bmx)[KA], ColState<T>& s, ColWork<T>& w, int* err,
                            int* err_k, int* err_it) {
  column_cell_phase<T, M>(CT, mth, K, dt, rdt, s, w);
  column_transport_phase<T>(C, fm, gr, K, dt, hdt2, sdt3, itelim, bmn, bmx, s, w, err, err_k, err_it);
}

template <class T>
__device__ void column_transport_phase(const Consts& C, const FastMath& fm, const double* gr, int K, double dt,
                                       double hdt2, double sdt3, int itelim, const int (*bmn)[KA],
                                       const int (*bmx)[KA], ColState<T>& s, ColWork<T>& w, int* err, int* err_k,
                                       int* err_it) {
  const int kmin = 1, kmax = K - 2;
  const double* gzh = gr + GF_GZH * K;
  const double* gzs = gr + GF_GZSHIFT * K;
  const double* dgz = gr + GF_DGZ * K;
  const double* dgzh = gr + GF_DGZH * K;
  const double* rdgz = gr + GF_RDGZ * K;
  const double* rdgzh = gr + GF_RDGZH * K;
  const double* afact = gr + GF_AFACT * K;
  const double* bfact = gr + GF_BFACT * K;
  const double* cfact = gr + GF_CFACT * K;
  const double* dfact = gr + GF_DFACT * K;
  const double* rdzs = gr + GF_RDZS * K;
  const double* rdzsh = gr + GF_RDZSH * K;

  // ---- departure distances (vadv1d_prep)
  for (int r = 0; r < 6; ++r) {
    const int t = r % 3, half = r / 3;
    const int mkmin = half ? kmin + 1 : kmin;
    const T* col = w.vt[t];
    for (int k = 0; k < K; ++k) {
      T z = T(0.0);
      if (k >= mkmin && k <= kmax) {
        if (!half) {
          auto wp = [&](int j) { return col[j]; };
          z = vadv_zdis<T>(wp, rdgz, rdzs, k, mkmin, kmax, T(dt), T(hdt2), T(sdt3));
        } else {
          auto wp = [&](int j) {
            return (j >= kmin + 1 && j <= kmax - 1) ? T(0.5) * (col[j] + col[j - 1]) : T(0.0);
          };
          z = vadv_zdis<T>(wp, rdgzh, rdzsh, k, mkmin, kmax, T(dt), T(hdt2), T(sdt3));
        }
      }
      w.zdis[r][k] = z;
    }
  }

  // ---- metric factors, kinetic energy, zeroed accumulators
  for (int k = 0; k < K; ++k) {
    w.drhoe[k] = w.drhophi[k] = w.dkinh[k] = w.dkinv[k] = T(0.0);
    w.drhogu[k] = w.drhogv[k] = w.drhogw[k] = T(0.0);
    w.dq[0][k] = w.dq[1][k] = w.dq[2][k] = T(0.0);
    w.rgs[k] = T(0.0);
    w.kinh[k] = T(0.0);
    w.kinv[k] = T(0.0);
    const bool interior = (k >= kmin && k <= kmax);
    if (interior) w.rgs[k] = s.gam2[k] / s.gsgam2[k];
    w.vi[k] = s.vx[k] * s.ix + s.vy[k] * s.iy + s.vz[k] * s.iz;
    w.vj[k] = s.vx[k] * s.jx + s.vy[k] * s.jy + s.vz[k] * s.jz;
    if (interior)
      w.kinh[k] = 0.5 * (s.rhogvx[k] * s.rhogvx[k] + s.rhogvy[k] * s.rhogvy[k] + s.rhogvz[k] * s.rhogvz[k]) / s.rhog[k];
    if (k >= kmin + 1 && k <= kmax) {
      const T c2w0 = afact[k] / s.gsgam2[k] * s.gsgam2h[k];
      const T c2w1 = bfact[k] / s.gsgam2[k - 1] * s.gsgam2h[k];
      const T rw = s.rhogw[k];
      w.kinv[k] = 0.5 * (rw * rw) / (c2w0 * s.rhog[k] + c2w1 * s.rhog[k - 1]);
    }
  }

  // ---- sedimentation of QR, QS, QG
  T acc[6] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
  const int tracer[3] = {I_QR, I_QS, I_QG};
  for (int t = 0; t < 3; ++t) {
    const int nq = tracer[t];
    const T* zdis0 = w.zdis[t];
    const T* zdis0h = w.zdis[3 + t];
    for (int k = 0; k < K; ++k) {
      w.base[k] = s.rhogq[nq][k] * w.rgs[k];
      if (k >= kmin && k <= kmax)
        w.kc[k] = (unsigned char)departure_cell_t(gzh, k, val(zdis0[k]), bmn[t][k], bmx[t][k], kmin, kmax);
    }
    for (int f = 0; f < 6; ++f) {
      for (int k = 0; k < K; ++k) {
        const T b = w.base[k];
        T r;
        switch (f) {
          case 0: r = b; break;
          case 1: r = b * CVDRY * s.tem[k]; break;
          case 2: r = b * GRAV * s.z[k]; break;
          case 3: r = s.q[nq][k] * w.rgs[k] * w.kinh[k]; break;
          case 4: r = b * w.vi[k]; break;
          default: r = b * w.vj[k]; break;
        }
        w.rhof[k] = r;
      }
      for (int k = 0; k < K; ++k) {
        T fl = T(0.0);
        if (k >= kmin && k <= kmax) fl = flux_integral_t(w.rhof, dgz, k, w.kc[k], zdis0[k], bmn[t][k], bmx[t][k]);
        w.f[k] = fl;
      }
      for (int k = kmin; k <= kmax; ++k) {
        const T fk = w.f[k], fk1 = w.f[k + 1];
        const T d = (fk1 - fk) * rdgz[k];
        switch (f) {
          case 0:
            w.dq[t][k] = -d;
            if (nq == I_QR) s.GPREC[k] = 0.0 + (-fk / dt);
            break;
          case 1: w.drhoe[k] = w.drhoe[k] - d; break;
          case 2: w.drhophi[k] = w.drhophi[k] - d; break;
          case 3: w.dkinh[k] = w.dkinh[k] - d; break;
          case 4: w.drhogu[k] = w.drhogu[k] - d; break;
          default: w.drhogv[k] = w.drhogv[k] - d; break;
        }
        if (k == kmin) {
          switch (f) {
            case 0:
              if (nq == I_QR) {
                acc[0] = acc[0] - fk / dt;
              } else {
                acc[1] = acc[1] - fk / dt;
                acc[2] = acc[2] + fk * LHF0 / dt;
              }
              break;
            case 1: acc[3] = acc[3] - fk / dt; break;
            case 2: acc[4] = acc[4] - fk / dt; break;
            case 3: acc[5] = acc[5] - fk / dt; break;
            default: break;
          }
        }
      }
    }
    // half levels
    for (int k = 0; k < K; ++k) {
      T qh = T(0.0);
      if (k >= kmin + 1 && k <= kmax) {
        qh = 0.5 * (s.q[nq][k] + s.q[nq][k - 1]) * (s.gam2h[k] / s.gsgam2h[k]);
        w.kc[k] = (unsigned char)departure_cell_t(gzs, k, val(zdis0h[k]), bmn[3 + t][k], bmx[3 + t][k], kmin + 1,
                                                  kmax);
      }
      w.base[k] = qh;
      w.rhof[k] = qh * w.kinv[k];
    }
    for (int wq = 0; wq < 2; ++wq) {
      for (int k = 0; k < K; ++k) {
        T fl = T(0.0);
        if (k >= kmin + 1 && k <= kmax)
          fl = flux_integral_t(w.rhof, dgzh, k, w.kc[k], zdis0h[k], bmn[3 + t][k], bmx[t][k]);
        w.f[k] = fl;
      }
      for (int k = 0; k < K; ++k) {
        if (k >= kmin + 1 && k <= kmax) {
          const T d = (w.f[k] - w.f[k - 1]) * rdgzh[k];
          if (wq == 0) w.dkinv[k] = w.dkinv[k] - d;
          else w.drhogw[k] = w.drhogw[k] - d;
        }
      }
      if (wq == 0)
        for (int k = 0; k < K; ++k) w.rhof[k] = (k >= kmin + 1 && k <= kmax) ? w.base[k] * s.rhogw[k] : T(0.0);
    }
  }

  // ---- apply the tendencies
  for (int k = 0; k < K; ++k) {
    const T dqr = w.dq[0][k], dqs = w.dq[1][k], dqg = w.dq[2][k];
    T rhoge = s.rhoge[k] + w.drhoe[k] + w.drhophi[k];
    w.kinh[k] = w.kinh[k] + w.dkinh[k];
    w.kinv[k] = w.kinv[k] + w.dkinv[k];
    const T du = w.drhogu[k], dv = w.drhogv[k];
    s.rhogvx[k] = s.rhogvx[k] + du * s.ix + dv * s.jx;
    s.rhogvy[k] = s.rhogvy[k] + du * s.iy + dv * s.jy;
    s.rhogvz[k] = s.rhogvz[k] + du * s.iz + dv * s.jz;
    const T rw = s.rhogw[k] + w.drhogw[k];
    s.rhogw[k] = rw;
    T rhog = s.rhog[k];
    const T zz = s.z[k];
    s.rhogq[I_QV][k] = s.rhogq[I_QV][k] + 0.0;
    s.rhogq[I_QC][k] = s.rhogq[I_QC][k] + 0.0;
    s.rhogq[I_QR][k] = s.rhogq[I_QR][k] + dqr;
    rhog = rhog + dqr;
    rhoge = rhoge - dqr * GRAV * zz;
    s.rhogq[I_QI][k] = s.rhogq[I_QI][k] + 0.0;
    s.rhogq[I_QS][k] = s.rhogq[I_QS][k] + dqs;
    rhog = rhog + dqs;
    rhoge = rhoge - dqs * GRAV * zz;
    s.rhogq[I_QG][k] = s.rhogq[I_QG][k] + dqg;
    rhog = rhog + dqg;
    rhoge = rhoge - dqg * GRAV * zz;
    s.rhog[k] = rhog;
    s.rhoge[k] = rhoge;
  }

  // ---- KIN2EIN: kinetic energy before (drhoe) and vertical energy after (drhophi)
  for (int k = 0; k < K; ++k) {
    w.drhoe[k] = T(0.0);
    w.drhophi[k] = T(0.0);
    if (k >= kmin && k <= kmax) {
      const T gh = s.gsgam2h[k + 1], rgh = 1.0 / gh;
      const T w2c0 = div_rn(cfact[k] * s.gsgam2[k], gh, rgh);
      const T w2c1 = div_rn(dfact[k] * s.gsgam2[k], gh, rgh);
      w.drhoe[k] = w.kinh[k] + (w2c0 * w.kinv[k + 1] + w2c1 * w.kinv[k]);
    }
    if (k >= kmin + 1 && k <= kmax) {
      const T c2w0 = afact[k] / s.gsgam2[k] * s.gsgam2h[k];
      const T c2w1 = bfact[k] / s.gsgam2[k - 1] * s.gsgam2h[k];
      const T rw = s.rhogw[k];
      w.drhophi[k] = 0.5 * (rw * rw) / (c2w0 * s.rhog[k] + c2w1 * s.rhog[k - 1]);
    }
  }

  // ---- per cell: KIN2EIN, thermodynamics, saturation adjustment, negative filter
  for (int k = 0; k < K; ++k) {
    const bool interior = (k >= kmin && k <= kmax);
    const T rhog = s.rhog[k];
    const T rrhog = 1.0 / rhog;
    T rhoge = s.rhoge[k];
    if (interior) {
      const T rvx = s.rhogvx[k], rvy = s.rhogvy[k], rvz = s.rhogvz[k];
      const T tmp_h = div_rn(0.5 * (rvx * rvx + rvy * rvy + rvz * rvz), rhog, rrhog);
      const T gh = s.gsgam2h[k + 1], rgh = 1.0 / gh;
      const T w2c0 = div_rn(cfact[k] * s.gsgam2[k], gh, rgh);
      const T w2c1 = div_rn(dfact[k] * s.gsgam2[k], gh, rgh);
      const T tmp = tmp_h + (w2c0 * w.drhophi[k + 1] + w2c1 * w.drhophi[k]);
      rhoge = rhoge + (w.drhoe[k] - tmp);
    }
    T rq[6], q[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) rq[n] = s.rhogq[n][k];
#pragma unroll
    for (int n = 0; n < 6; ++n) q[n] = div_rn(rq[n], rhog, rrhog);
    const T gsg = s.gsgam2[k];
    T rho = rhog / gsg;
    const T ein = div_rn(rhoge, rhog, rrhog);
    T qd = T(1.0);
#pragma unroll
    for (int n = 1; n <= 5; ++n) qd = qd - q[n];
    T cvt = T(0.0), qdl = T(1.0);
#pragma unroll
    for (int n = 1; n <= 5; ++n) {
      cvt = cvt + q[n] * CVDRY;
      qdl = qdl - q[n];
    }
    cvt = cvt + qdl * CVDRY;
    T tem = ein / cvt;
    T pre = rho * tem * (qdl * RDRY + q[I_QV] * RVAP);
    const T ein_moist = ein + q[I_QV] * LHV0;
    const T qsum = q[I_QV] + q[I_QC];
    q[I_QV] = qsum;
    q[I_QC] = T(0.0);
    T cvtot = qd * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cvtot = cvtot + q[n] * CVDRY;
    const T rho_l = rho;
    tem = (ein_moist - q[I_QV] * LHV0) / cvtot;
    if (interior) {
      int iters = 0;
      const int rc = satadjust_t(C, fm, itelim, ein_moist, qsum, rho_l, q, tem, &iters);
      if (rc != 0 && *err == 0) {
        *err = rc;
        *err_k = k;
        *err_it = iters;
      }
    }
    rq[I_QV] = rhog * q[I_QV];
    rq[I_QC] = rhog * q[I_QC];
    cvtot = qd * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cvtot = cvtot + q[n] * CVDRY;
    rhoge = rhog * tem * cvtot;
    T rhog_o = rhog;
    if (interior) {
      T diffq = T(0.0);
#pragma unroll
      for (int n = 2; n <= 5; ++n) {
        diffq += rq[n];
        rq[n] = dmax(rq[n], T(0.0));
      }
#pragma unroll
      for (int n = 2; n <= 5; ++n) diffq -= rq[n];
      rq[I_QV] += diffq;
      diffq = rq[I_QV];
      rq[I_QV] = dmax(rq[I_QV], T(0.0));
      diffq -= rq[I_QV];
      rhog_o = rhog * (1.0 - diffq);
      rho = rhog_o / gsg;
      const T rrhog_o = 1.0 / rhog_o;
#pragma unroll
      for (int n = 1; n <= 5; ++n) q[n] = div_rn(rq[n], rhog_o, rrhog_o);
      T qdf = T(1.0);
#pragma unroll
      for (int n = 1; n <= 5; ++n) qdf = qdf - q[n];
      T cva = qdf * CVDRY;
#pragma unroll
      for (int n = 1; n <= 5; ++n) cva = cva + q[n] * CVDRY;
      rhoge = tem * rhog_o * cva;
      pre = rho * (qdf * RDRY + q[I_QV] * RVAP) * tem;
    }
    s.rhog[k] = rhog_o;
    s.rhoge[k] = rhoge;
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      s.rhogq[n][k] = rq[n];
      s.q[n][k] = q[n];
    }
    s.rho[k] = rho;
    s.tem[k] = tem;
    s.pre[k] = pre;
    s.qd[k] = qd;
    if (!interior) {
      s.GPREC[k] = T(0.0);
      s.re_liquid[k] = T(0.0);
      s.re_cld[k] = T(0.0);
    }
  }
  s.precip0 = 0.0 + acc[0];
  s.precip1 = 0.0 + acc[1];
  s.lh_heat = 0.0 + acc[2];
  s.p_rhoe = 0.0 + acc[3];
  s.p_rhophi = 0.0 + acc[4];
  s.p_rhokin = 0.0 + acc[5];
}

}  // namespace nsw6
