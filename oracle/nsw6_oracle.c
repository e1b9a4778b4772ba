/* CPU restatement of one NICAM NSW6 microphysics step (TEST INFRASTRUCTURE ONLY).
 *
 * Restates the reference's Kokkos code path pass by pass; every function and
 * block cites the reference source (path:line) it follows.  Expressions keep
 * the reference's evaluation order so that, compiled without floating-point
 * contraction and linked against the same libm, the results equal the
 * reference build bit for bit.  See nsw6_oracle.h.
 */
#include "nsw6_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Phase markers for the operation-counting build (oracle/opcount.cpp); empty
 * otherwise.  Phase 1: negative filter, saturation values, process rates and
 * cell updates (the GPU cell kernel); phase 2: transport, saturation
 * adjustment and closing filter (the GPU column kernel); phase 3: the
 * departure distances of vadv1d_prep (computed in the GPU cell kernel). */
#ifndef NSW6O_PHASE
#define NSW6O_PHASE(n)
#endif

/* Decision-site markers for the decision-recording build
 * (oracle/branchsig.cpp), which tags every discrete decision of the step with
 * the part of the algorithm that takes it; empty otherwise. */
#ifndef NSW6O_SITE
#define NSW6O_SITE(n)
#endif
enum {
  SITE_OTHER,      /* thermodynamics, updates, metric factors */
  SITE_RATES,      /* process rates, slope parameters, fall speeds (TagBigLoop) */
  SITE_LIMITER,    /* the rate limiters and per-species loss limiters, :1249-1559 */
  SITE_NEGFILTER,  /* negative_filter */
  SITE_DEPARTURE,  /* vadv1d_prep: region-wide extrema, flux bounds, departure cells */
  SITE_FLUXSUM,    /* vadv1d_getflux_new: the flux integral's weights */
  SITE_EPSFILTER,  /* vadv1d_getflux_new: the |flux| < EPS filter */
  SITE_NEWTON,     /* SATURATION_adjustment: saturation test and Newton iteration */
  SITE_DIAG        /* effective radii and cloud top */
};

#ifdef _OPENMP
#include <omp.h>
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

/* ------------------------------------------------------------------ constants
 * include/problemsize.h:86-135 and the private constants of the modules. */
#define CONST_PI 3.141592653589793
#define CONST_EPS 2.220446E-16
#define CONST_UNDEF (-9.9999E+30)
#define CONST_GRAV 9.79764
#define CONST_Rdry 287.04
#define CONST_CVdry 717.56
#define CONST_Rvap 461.46
#define CONST_CL 4218.0
#define CONST_PSAT0 610.7
#define CONST_LHV0 2501000.0
#define CONST_LHS0 2834000.0
#define CONST_LHF0 333000.0
#define CONST_Pstd 101325.0
#define CONST_TEM00 273.15
#define CONST_DWATR 1000.0
#define TEM_MIN 10.0 /* mod_satadjust.cpp:6 */
#define DENS00 1.28  /* mod_mp_nsw6.cpp:8 */
#define NQ 6
#define I_QV 0
#define I_QC 1
#define I_QR 2
#define I_QI 3
#define I_QS 4
#define I_QG 5
#define NQW_STR 1
#define NQW_END 5

/* Argument positions of mp_driver (mod_mp_driver.h:71-124). */
enum {
  A_rhog, A_rhogvx, A_rhogvy, A_rhogvz, A_rhogw, A_rhoge, A_rhogq, A_vx, A_vy, A_vz, A_w,
  A_unccn, A_rho, A_tem, A_pre, A_q, A_qd, A_precip, A_ISO1, A_ISO2, A_precip_rhoe,
  A_precip_lh_heat, A_precip_rhophi, A_precip_rhokin, A_re_liquid, A_re_solid, A_re_cld,
  A_rctop, A_rwtop, A_tctop, A_frhoge_af, A_frhogqv_af, A_frhoge_rad, A_rhogqke, A_gsgam2,
  A_gsgam2h, A_gam2, A_gam2h, A_ix, A_iy, A_iz, A_jx, A_jy, A_jz, A_z, A_zh, A_GDCLW,
  A_GDCFRC, A_GPREC, A_CBMFX, A_COUNT
};

static inline double dmin(double a, double b) { return (b < a) ? b : a; }  /* Kokkos::min */
static inline double dmax(double a, double b) { return (a < b) ? b : a; }  /* Kokkos::max */

void nsw6o_default_params(nsw6o_params* p) {
  p->beta_saut = 5.0E-3;   /* PSAUT_BETA0 in mp_nsw6_init, mod_mp_nsw6.cpp:287-294 */
  p->qicrt_saut = 0.0;     /* mod_mp_nsw6.h:87 */
  p->Cr = 130.0;           /* mod_mp_nsw6.h:27 */
  p->Cs = 4.84;            /* mod_mp_nsw6.h:28 */
  /* Cg = sqrt(4 rho_g GRAV / (3 dens00 C_d)), mod_mp_nsw6.cpp:337 */
  p->Cg = sqrt((4.0 * 400.0 * CONST_GRAV) / (3.0 * DENS00 * 0.6));
  p->ice_nuc = 4.92E-11;   /* mod_mp_nsw6.cpp:1083 */
  p->kk_aut = 1350.0;      /* mod_mp_nsw6.cpp:1154 */
}

int nsw6o_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ gamma
 * MISC_gammafunc, mod_debug.cpp:332-361 (Lanczos series, 6 coefficients). */
static double gammafunc(double xx) {
  static const double coef[6] = {+76.18009172947146, -86.50532032941677, +24.01409824083091,
                                 -1.231739572450155, +0.1208650973866179E-2, -0.5395239384953E-5};
  double x = xx, y = x, tmp = x + 5.5;
  tmp = tmp - (x + 0.5) * log(tmp);
  double ser = 1.000000000190015;
  for (int j = 0; j < 6; ++j) {
    y += 1;
    ser += coef[j] / y;
  }
  return exp(-tmp + log(2.5066282746310005 * ser / x));
}

/* ------------------------------------------------------------------ scheme constants
 * mp_nsw6_init (mod_mp_nsw6.cpp:276-434) with the settings it hard-wires
 * (Roh & Satoh 2014 snow, explicit ice generation, KK2000, beta_gaut = 0),
 * the struct defaults of GlobalParams (mod_mp_nsw6.h:16-123) and the
 * effective-radius constants of mp_nsw6_new::init (mod_mp_nsw6.cpp:506-517). */
typedef struct {
  double Ar, As, Ag, Cr, Cs, Cg, N0r, N0s, N0g;
  double GAM, GAM_2, GAM_3, GAM_1br, GAM_2br, GAM_3br, GAM_3dr, GAM_6dr, GAM_1brdr, GAM_5dr_h;
  double GAM_1bs, GAM_2bs, GAM_3bs, GAM_3ds, GAM_1bsds, GAM_5ds_h;
  double GAM_1bg, GAM_3dg, GAM_1bgdg, GAM_5dg_h;
  double Eiw, Erw, Esw, Egw, Eri, Esi, Egi, Esr, Egr, Egs, gamma_sacr, gamma_gacs, mi;
  double beta_saut, gamma_saut, beta_gaut, gamma_gaut, qicrt_saut, qscrt_gaut;
  double f1r, f2r, f1s, f2s, f1g, f2g, A_frz, B_frz, mi40, mi50, vti50, Ri50;
  double sw_expice, Nc_ihtr, Di_max, Di_a, sw_kk2000, sw_constVti, CONST_Vti, sw_roh2014, ln10;
  double coef_a[10], coef_b[10];
  double Nc_def, coef_dgam, coef_xf;
  double ice_nuc, kk_aut;
  double LovR_liq, LovR_ice, CPovR_liq, CPovR_ice, CVovR_liq, RTEM00;
} consts_t;

static void make_consts(consts_t* c, const nsw6o_params* p) {
  static const double ca[10] = {5.065339, -0.062659, -3.032362, 0.029469, -0.000285,
                                0.31255, 0.000204, 0.003199, 0.0, -0.015952};
  static const double cb[10] = {0.476221, -0.015896, 0.165977, 0.007468, -0.000141,
                                0.060366, 0.000079, 0.000594, 0.0, -0.003577};
  memset(c, 0, sizeof(*c));
  const double rho_s = 100.0, rho_g = 400.0;
  double Br = 3.0, Bs = 3.0, Bg = 3.0, Dr = 0.50, Ds = 0.25, Dg = 0.50;
  c->N0r = 8.E+6;
  c->N0s = 3.E+6;
  c->Ar = CONST_PI * CONST_DWATR / 6.0;
  c->As = CONST_PI * rho_s / 6.0;
  c->Ag = CONST_PI * rho_g / 6.0;
  /* Roh and Satoh (2014) block, mod_mp_nsw6.cpp:345-356 */
  c->sw_roh2014 = 1.0;
  c->N0g = 4.0E+8;
  c->As = 0.069;
  Bs = 2.0;
  c->Eiw = 1.0; c->Erw = 1.0; c->Esw = 1.0; c->Egw = 1.0; c->Eri = 1.0;
  c->Esi = 0.25; c->Egi = 0.0; c->Esr = 1.0; c->Egr = 1.0; c->Egs = 0.0;
  c->gamma_sacr = 6.0E-2;  /* mod_mp_nsw6.cpp:286 */
  c->gamma_gacs = 90.E-3;
  c->mi = 4.19E-13;
  c->beta_saut = p->beta_saut;
  c->gamma_saut = 6.0E-2;  /* mod_mp_nsw6.cpp:288 */
  c->beta_gaut = 0.0;      /* INC_PGAUT = false, mod_mp_nsw6.cpp:394-397 */
  c->gamma_gaut = 90.E-3;
  c->qicrt_saut = p->qicrt_saut;
  c->qscrt_gaut = 6.E-4;
  c->f1r = 0.78; c->f2r = 0.27; c->f1s = 0.65; c->f2s = 0.39; c->f1g = 0.78; c->f2g = 0.27;
  c->A_frz = 0.66; c->B_frz = 100.0;
  c->mi40 = 2.46E-10; c->mi50 = 4.80E-10; c->vti50 = 1.0; c->Ri50 = 5.E-5;
  c->sw_expice = 1.0;      /* OPT_EXPLICIT_ICEGEN, mod_mp_nsw6.cpp:364-368 */
  c->Nc_ihtr = 300.0; c->Di_max = 500.E-6; c->Di_a = 11.9;
  c->sw_kk2000 = 1.0;      /* mod_mp_nsw6.cpp:382-386 */
  c->CONST_Vti = CONST_UNDEF;
  c->sw_constVti = 0.0;    /* CONST_Vti == UNDEF, mod_mp_nsw6.cpp:399-407 */
  c->Cr = p->Cr;
  c->Cs = p->Cs;
  c->Cg = p->Cg;
  c->GAM = 1.0; c->GAM_2 = 1.0; c->GAM_3 = 2.0;
  c->GAM_1br = gammafunc(1.0 + Br);
  c->GAM_2br = gammafunc(2.0 + Br);
  c->GAM_3br = gammafunc(3.0 + Br);
  c->GAM_3dr = gammafunc(3.0 + Dr);
  c->GAM_6dr = gammafunc(6.0 + Dr);
  c->GAM_1brdr = gammafunc(1.0 + Br + Dr);
  c->GAM_5dr_h = gammafunc(0.5 * (5.0 + Dr));
  c->GAM_1bs = gammafunc(1.0 + Bs);
  c->GAM_2bs = gammafunc(2.0 + Bs);
  c->GAM_3bs = gammafunc(3.0 + Bs);
  c->GAM_3ds = gammafunc(3.0 + Ds);
  c->GAM_1bsds = gammafunc(1.0 + Bs + Ds);
  c->GAM_5ds_h = gammafunc(0.5 * (5.0 + Ds));
  c->GAM_1bg = gammafunc(1.0 + Bg);
  c->GAM_3dg = gammafunc(3.0 + Dg);
  c->GAM_1bgdg = gammafunc(1.0 + Bg + Dg);
  c->GAM_5dg_h = gammafunc(0.5 * (5.0 + Dg));
  c->ln10 = log(10.0);
  memcpy(c->coef_a, ca, sizeof(ca));
  memcpy(c->coef_b, cb, sizeof(cb));
  c->Nc_def = 50.0;        /* Nc_ocn, mod_mp_nsw6.cpp:281 */
  {
    double Dc = 0.146 - 5.964E-2 * log(c->Nc_def / 2000.0);
    double dgamma_a = 0.1444 / (Dc * Dc);
    double GAM_dgam = gammafunc(dgamma_a);
    double GAM_dgam23 = gammafunc(dgamma_a + 2.0 / 3.0);
    c->coef_dgam = GAM_dgam23 / GAM_dgam * pow(dgamma_a, (-2.0 / 3.0));
    c->coef_xf = 3.0 / 4.0 / CONST_PI / CONST_DWATR;
  }
  c->ice_nuc = p->ice_nuc;
  c->kk_aut = p->kk_aut;
  /* SATURATION_Setup with EIN_TYPE = "SIMPLE", mod_satadjust.cpp:24-47 */
  c->CPovR_liq = 0.0;
  c->CPovR_ice = 0.0;
  c->CVovR_liq = 0.0;
  c->LovR_liq = CONST_LHV0 / CONST_Rvap;
  c->LovR_ice = CONST_LHS0 / CONST_Rvap;
  c->RTEM00 = 1.0 / CONST_TEM00;
}

/* ------------------------------------------------------------------ grid
 * GRD_Setup, mod_debug.cpp:92-187. */
typedef struct {
  double *gz, *gzh, *dgz, *dgzh, *rdgz, *rdgzh, *afact, *bfact, *cfact, *dfact, *gz_shift;
} grid_t;

static void make_grid(grid_t* g, int K, const double* gz, const double* gzh, double* mem) {
  g->gz = mem;
  g->gzh = mem + K;
  g->dgz = mem + 2 * K;
  g->dgzh = mem + 3 * K;
  g->rdgz = mem + 4 * K;
  g->rdgzh = mem + 5 * K;
  g->afact = mem + 6 * K;
  g->bfact = mem + 7 * K;
  g->cfact = mem + 8 * K;
  g->dfact = mem + 9 * K;
  g->gz_shift = mem + 10 * K;
  memset(mem, 0, sizeof(double) * 11 * (size_t)K);
  const int kmin = 1, kmax = K - 2;
  for (int k = 0; k < K; ++k) {
    g->gz[k] = gz[k];
    g->gzh[k] = gzh[k];
  }
  for (int k = kmin - 1; k <= kmax; ++k) g->dgz[k] = g->gzh[k + 1] - g->gzh[k];
  g->dgz[kmax + 1] = g->dgz[kmax];
  for (int k = kmin; k <= kmax + 1; ++k) g->dgzh[k] = g->gz[k] - g->gz[k - 1];
  g->dgzh[kmin - 1] = g->dgzh[kmin];
  for (int k = 0; k < K; ++k) {
    g->rdgz[k] = 1.0 / g->dgz[k];
    g->rdgzh[k] = 1.0 / g->dgzh[k];
  }
  for (int k = kmin; k <= kmax + 1; ++k)
    g->afact[k] = (g->gzh[k] - g->gz[k - 1]) / (g->gz[k] - g->gz[k - 1]);
  g->afact[kmin - 1] = 1.0;
  for (int k = 0; k < K; ++k) g->bfact[k] = 1.0 - g->afact[k];
  for (int k = kmin; k <= kmax; ++k)
    g->cfact[k] = (g->gz[k] - g->gzh[k]) / (g->gzh[k + 1] - g->gzh[k]);
  g->cfact[kmin - 1] = 1.0;
  g->cfact[kmax + 1] = 0.0;
  for (int k = 0; k < K; ++k) g->dfact[k] = 1.0 - g->cfact[k];
  /* GRD_gz_shift, mod_precip_transport.cpp:698-709 (k = 0 stays zero) */
  for (int k = kmin; k <= kmax + 1; ++k) g->gz_shift[k] = g->gz[k - 1];
}

/* ------------------------------------------------------------------ work space */
typedef struct {
  int G, K, kmin, kmax;
  size_t N; /* K*G */
} dims_t;

#define IX(k, g) ((size_t)(k) * (size_t)D->G + (size_t)(g))
#define QX(nq, k, g) (((size_t)(nq) * (size_t)D->K + (size_t)(k)) * (size_t)D->G + (size_t)(g))

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* THRMDYN_qd, mod_thrmdyn.cpp:98-113 (all k). */
static void thrmdyn_qd(const dims_t* D, const double* q, double* qd) {
  OMP_FOR
  for (size_t i = 0; i < D->N; ++i) {
    double v = 1.0;
    for (int nq = NQW_STR; nq <= NQW_END; ++nq) v = v - q[(size_t)nq * D->N + i];
    qd[i] = v;
  }
}

/* THRMDYN_cv, mod_thrmdyn.cpp:115-135 (all k; CVW = CVdry for every tracer,
 * CVW_CPW_Setup mod_debug.cpp:76-90). */
static void thrmdyn_cv(const dims_t* D, const double* qd, const double* q, double* cv) {
  OMP_FOR
  for (size_t i = 0; i < D->N; ++i) {
    double v = qd[i] * CONST_CVdry;
    for (int nq = NQW_STR; nq <= NQW_END; ++nq) v = v + q[(size_t)nq * D->N + i] * CONST_CVdry;
    cv[i] = v;
  }
}

/* negative_filter, mod_mp_nsw6.cpp:1750-1832 (interior levels). */
static void negative_filter(const dims_t* D, double* rhog, double* rhoge, double* rhogq, double* rho,
                            const double* tem, double* pre, double* q, const double* gsgam2,
                            double* qd_w, double* cv_w) {
  const size_t lo = IX(D->kmin, 0), hi = IX(D->kmax + 1, 0), N = D->N;
  NSW6O_SITE(SITE_NEGFILTER);
  OMP_FOR
  for (size_t i = lo; i < hi; ++i) {
    double diffq = 0.0;
    for (int nq = NQW_STR + 1; nq <= NQW_END; ++nq) {
      diffq += rhogq[nq * N + i];
      rhogq[nq * N + i] = dmax(rhogq[nq * N + i], 0.0);
    }
    for (int nq = NQW_STR + 1; nq <= NQW_END; ++nq) diffq -= rhogq[nq * N + i];
    rhogq[I_QV * N + i] += diffq;
  }
  OMP_FOR
  for (size_t i = lo; i < hi; ++i) {
    double diffq = rhogq[I_QV * N + i];
    rhogq[I_QV * N + i] = dmax(rhogq[I_QV * N + i], 0.0);
    diffq -= rhogq[I_QV * N + i];
    rhog[i] = rhog[i] * (1.0 - diffq);
    rho[i] = rhog[i] / gsgam2[i];
  }
  for (int nq = NQW_STR; nq <= NQW_END; ++nq) {
    OMP_FOR
    for (size_t i = lo; i < hi; ++i) q[nq * N + i] = rhogq[nq * N + i] / rhog[i];
  }
  thrmdyn_qd(D, q, qd_w);
  thrmdyn_cv(D, qd_w, q, cv_w);
  OMP_FOR
  for (size_t i = lo; i < hi; ++i) {
    rhoge[i] = tem[i] * rhog[i] * cv_w[i];
    pre[i] = rho[i] * (qd_w[i] * CONST_Rdry + q[I_QV * N + i] * CONST_Rvap) * tem[i];
  }
  NSW6O_SITE(SITE_OTHER);
}

/* SATURATION_psat_liq / _ice, mod_satadjust.cpp:80-106, 133-160 (all k). */
static void psat_fn(const dims_t* D, const consts_t* c, const double* tem, double* psat, double CPovR,
                    double LovR) {
  OMP_FOR
  for (size_t i = 0; i < D->N; ++i) {
    double rtem = 1.0 / (dmax(tem[i], TEM_MIN));
    psat[i] = CONST_PSAT0 * pow((tem[i] * c->RTEM00), CPovR) * exp(LovR * (c->RTEM00 - rtem));
  }
}

/* Bergeron_param, mod_mp_nsw6.cpp:1834-1890 (interior levels).  The
 * interpolation weight is fact = -(temc + itemc - 1), as in the reference. */
static void bergeron(const dims_t* D, const double* tem, double* a1, double* a2, double* ma2) {
  NSW6O_SITE(SITE_RATES);
  static const double a1_tab[32] = {
      0.0001E-7, 0.7939E-7, 0.7841E-6, 0.3369E-5, 0.4336E-5, 0.5285E-5, 0.3728E-5, 0.1852E-5,
      0.2991E-6, 0.4248E-6, 0.7434E-6, 0.1812E-5, 0.4394E-5, 0.9145E-5, 0.1725E-4, 0.3348E-4,
      0.1725E-4, 0.9175E-5, 0.4412E-5, 0.2252E-5, 0.9115E-6, 0.4876E-6, 0.3473E-6, 0.4758E-6,
      0.6306E-6, 0.8573E-6, 0.7868E-6, 0.7192E-6, 0.6513E-6, 0.5956E-6, 0.5333E-6, 0.4834E-6};
  static const double a2_tab[32] = {
      0.0100, 0.4006, 0.4831, 0.5320, 0.5307, 0.5319, 0.5249, 0.4888, 0.3849, 0.4047, 0.4318,
      0.4771, 0.5183, 0.5463, 0.5651, 0.5813, 0.5655, 0.5478, 0.5203, 0.4906, 0.4447, 0.4126,
      0.3960, 0.4149, 0.4320, 0.4506, 0.4483, 0.4460, 0.4433, 0.4413, 0.4382, 0.4361};
  const size_t lo = IX(D->kmin, 0), hi = IX(D->kmax + 1, 0);
  OMP_FOR
  for (size_t i = lo; i < hi; ++i) {
    double temc = dmin(dmax(tem[i] - CONST_TEM00, -30.99), 0.0);
    int itemc = (int)(-temc);
    double fact = -(temc + (double)(itemc - 1));
    double v1 = (1.0 - fact) * a1_tab[itemc] + (fact)*a1_tab[itemc + 1];
    double v2 = (1.0 - fact) * a2_tab[itemc] + (fact)*a2_tab[itemc + 1];
    a2[i] = v2;
    ma2[i] = 1.0 - v2;
    a1[i] = v1 * pow(1.0E-3, ma2[i]);
  }
}

/* Process-rate indices of the reference's wk[] (mod_mp_nsw6.cpp:13-63). */
enum {
  I_dqv_dt, I_dqc_dt, I_dqr_dt, I_dqi_dt, I_dqs_dt, I_dqg_dt, I_delta1, I_delta2, I_spsati,
  I_iceflg, I_RLMDr, I_RLMDs, I_RLMDg, I_Piacr, I_Psacr, I_Praci, I_Pigen, I_Pidep, I_Psdep,
  I_Pgdep, I_Praut, I_Pracw, I_Pihom, I_Pihtr, I_Psacw, I_Psfw, I_Pgacw, I_Prevp, I_Piacr_s,
  I_Psacr_s, I_Piacr_g, I_Psacr_g, I_Pgacr, I_Pgfrz, I_Pisub, I_Pimlt, I_Psaut, I_Praci_s,
  I_Psaci, I_Psfi, I_Praci_g, I_Pgaci, I_Pssub, I_Psmlt, I_Pgaut, I_Pracs, I_Pgacs, I_Pgsub,
  I_Pgmlt, WK_NMAX
};

typedef struct {
  double drhogq[6]; /* v c r i s g */
  double Vt[4];     /* QR QI QS QG */
  double rceff, rceff_cld, rctop, tctop, rctop_cld, tctop_cld;
} bigloop_out_t;

/* mp_nsw6_new::operator()(TagBigLoop), mod_mp_nsw6.cpp:760-1594, for one cell. */
static void big_loop_cell(const consts_t* c, double dens, double temp, const double qin[6],
                          double qsatl, double qsati, double Nc, double a1, double a2, double ma2,
                          double pre, double rhog, double dt, bigloop_out_t* o) {
  double wk[WK_NMAX];
  const double EPS = CONST_EPS, PI = CONST_PI, UNDEF = CONST_UNDEF, Rvap = CONST_Rvap;
  const double LHV0 = CONST_LHV0, LHS0 = CONST_LHS0, LHF0 = CONST_LHF0, PRE00 = CONST_Pstd;
  const double Ka0 = 2.428E-2, dKa_dT = 7.47E-5, Kd0 = 2.222E-5, dKd_dT = 1.37E-7;
  const double nu0 = 1.718E-5, dnu_dT = 5.28E-8;
  const double r2_min = 1.0E-10, q_min = 1.0E-5;
  const double Ar = c->Ar, As = c->As, Ag = c->Ag, Cr = c->Cr, Cs = c->Cs, Cg = c->Cg;
  const double N0r = c->N0r, N0s = c->N0s, N0g = c->N0g;
  const double GAM = c->GAM, GAM_2 = c->GAM_2, GAM_3 = c->GAM_3;
  const double sw_roh2014 = c->sw_roh2014, ln10 = c->ln10, sw_expice = c->sw_expice;
  const double sw_kk2000 = c->sw_kk2000;

  NSW6O_SITE(SITE_RATES);
  double qv = dmax(qin[0], 0.0), qc = dmax(qin[1], 0.0), qr = dmax(qin[2], 0.0);
  double qi = dmax(qin[3], 0.0), qs = dmax(qin[4], 0.0), qg = dmax(qin[5], 0.0);

  /* :910-946 */
  double Sliq = qv / (dmax(qsatl, EPS));
  double Sice = qv / (dmax(qsati, EPS));
  double Rdens = 1.0 / dens;
  double rho_fact = sqrt(DENS00 * Rdens);
  double temc = temp - CONST_TEM00;
  wk[I_delta1] = (0.5 + copysign(0.5, qr - 1.0E-4));
  wk[I_delta2] = (0.5 + copysign(0.5, 1.0E-4 - qr)) * (0.5 + copysign(0.5, 1.0E-4 - qs));
  wk[I_spsati] = 0.5 + copysign(0.5, Sice - 1.0);
  wk[I_iceflg] = 0.5 - copysign(0.5, temc);
  wk[I_dqv_dt] = qv / dt;
  wk[I_dqc_dt] = qc / dt;
  wk[I_dqr_dt] = qr / dt;
  wk[I_dqi_dt] = qi / dt;
  wk[I_dqs_dt] = qs / dt;
  wk[I_dqg_dt] = qg / dt;
  double sw_bergeron = (0.5 + copysign(0.5, temc + 30.0)) * (0.5 + copysign(0.5, 0.0 - temc)) *
                       (1.0 - sw_expice);

  /* rain slope parameter, :953-967 */
  double zerosw = 0.5 - copysign(0.5, qr - 1.0E-12);
  double RLMDr = sqrt(sqrt(dens * qr / (Ar * N0r * c->GAM_1br) + zerosw)) * (1.0 - zerosw);
  double RLMDr_dr = sqrt(RLMDr);
  double RLMDr_2 = pow(RLMDr, 2);
  double RLMDr_3 = pow(RLMDr, 3);
  double RLMDr_7 = pow(RLMDr, 7);
  double RLMDr_1br = pow(RLMDr, 4);
  double RLMDr_2br = pow(RLMDr, 5);
  double RLMDr_3br = pow(RLMDr, 6);
  double RLMDr_3dr = pow(RLMDr, 3) * RLMDr_dr;
  double RLMDr_5dr = pow(RLMDr, 5) * RLMDr_dr;
  double RLMDr_6dr = pow(RLMDr, 6) * RLMDr_dr;

  /* snow slope parameter and moments, :969-992 */
  zerosw = 0.5 - copysign(0.5, qs - 1.0E-12);
  double RLMDs = sqrt(sqrt(dens * qs / (As * N0s * c->GAM_1bs) + zerosw)) * (1.0 - zerosw);
  double RLMDs_ds = sqrt(sqrt(RLMDs));
  double RLMDs_2 = pow(RLMDs, 2);
  double RLMDs_3 = pow(RLMDs, 3);
  double RLMDs_1bs = pow(RLMDs, 4);
  double RLMDs_2bs = pow(RLMDs, 5);
  double RLMDs_3bs = pow(RLMDs, 6);
  double RLMDs_3ds = pow(RLMDs, 3) * RLMDs_ds;
  double RLMDs_5ds = pow(RLMDs, 5) * RLMDs_ds;
  double MOMs_0 = N0s * GAM * RLMDs;
  double MOMs_1 = N0s * GAM_2 * RLMDs_2;
  double MOMs_2 = N0s * GAM_3 * RLMDs_3;
  double MOMs_0bs = N0s * c->GAM_1bs * RLMDs_1bs;
  double MOMs_1bs = N0s * c->GAM_2bs * RLMDs_2bs;
  double MOMs_2bs = N0s * c->GAM_3bs * RLMDs_3bs;
  double MOMs_2ds = N0s * c->GAM_3ds * RLMDs_3ds;
  double MOMs_5ds_h = N0s * c->GAM_5ds_h * sqrt(RLMDs_5ds);
  double RMOMs_Vt = c->GAM_1bsds / c->GAM_1bs * RLMDs_ds;

  /* Roh and Satoh (2014) bimodal snow moments, :994-1057 */
  double Xs2 = dens * qs / As;
  zerosw = 0.5 - copysign(0.5, Xs2 - 1.0E-12);
  double tems = dmin(-0.1, temc);
  const double* ca = c->coef_a;
  const double* cb = c->coef_b;
  double cat[4], cbt[4];
  cat[0] = ca[0] + tems * (ca[1] + tems * (ca[4] + tems * ca[8]));
  cat[1] = ca[2] + tems * (ca[3] + tems * ca[6]);
  cat[2] = ca[5] + tems * ca[7];
  cat[3] = ca[9];
  cbt[0] = cb[0] + tems * (cb[1] + tems * (cb[4] + tems * cb[8]));
  cbt[1] = cb[2] + tems * (cb[3] + tems * cb[6]);
  cbt[2] = cb[5] + tems * cb[7];
  cbt[3] = cb[9];
  double loga_, b_, nm;
  loga_ = cat[0];
  b_ = cbt[0];
  MOMs_0 = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) +
           (1.0 - sw_roh2014) * MOMs_0;
  nm = 1.0;
  loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  MOMs_1 = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) +
           (1.0 - sw_roh2014) * MOMs_1;
  MOMs_2 = sw_roh2014 * Xs2 + (1.0 - sw_roh2014) * MOMs_2;
  nm = 2.0;
  loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  MOMs_0bs = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) +
             (1.0 - sw_roh2014) * MOMs_0bs;
  nm = 3.0;
  loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  MOMs_1bs = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) +
             (1.0 - sw_roh2014) * MOMs_1bs;
  nm = 4.0;
  loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  MOMs_2bs = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) +
             (1.0 - sw_roh2014) * MOMs_2bs;
  nm = 2.25;
  loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  MOMs_2ds = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) +
             (1.0 - sw_roh2014) * MOMs_2ds;
  nm = 1.625;
  loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  MOMs_5ds_h = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) +
               (1.0 - sw_roh2014) * MOMs_5ds_h;
  nm = 2.25;
  loga_ = cat[0] + nm * (cat[1] + nm * (cat[2] + nm * cat[3]));
  b_ = cbt[0] + nm * (cbt[1] + nm * (cbt[2] + nm * cbt[3]));
  RMOMs_Vt = sw_roh2014 * exp(ln10 * loga_) * exp(log(Xs2 + zerosw) * b_) * (1.0 - zerosw) /
                 (MOMs_0bs + zerosw) +
             (1.0 - sw_roh2014) * RMOMs_Vt;

  /* graupel slope parameter, :1059-1066 */
  zerosw = 0.5 - copysign(0.5, qg - 1.0E-12);
  double RLMDg = sqrt(sqrt(dens * qg / (Ag * N0g * c->GAM_1bg) + zerosw)) * (1.0 - zerosw);
  double RLMDg_dg = sqrt(RLMDg);
  double RLMDg_2 = pow(RLMDg, 2);
  double RLMDg_3 = pow(RLMDg, 3);
  double RLMDg_3dg = pow(RLMDg, 3) * RLMDg_dg;
  double RLMDg_5dg = pow(RLMDg, 5) * RLMDg_dg;
  wk[I_RLMDr] = RLMDr;
  wk[I_RLMDs] = RLMDs;
  wk[I_RLMDg] = RLMDg;

  /* terminal velocity, :1072-1078 */
  zerosw = 0.5 - copysign(0.5, qi - 1.0E-8);
  double Vti = (1.0 - c->sw_constVti) * (-3.29) * exp(log(dens * qi + zerosw) * 0.16) * (1.0 - zerosw) +
               (c->sw_constVti) * (-c->CONST_Vti);
  double Vtr = -Cr * rho_fact * c->GAM_1brdr / c->GAM_1br * RLMDr_dr;
  double Vts = -Cs * rho_fact * RMOMs_Vt;
  double Vtg = -Cg * rho_fact * c->GAM_1bgdg / c->GAM_1bg * RLMDg_dg;

  /* nucleation, :1080-1085 */
  double Ni0 = dmax(exp(-0.1 * temc), 1.0) * 1000.0;
  double Qi0 = c->ice_nuc * exp(log(Ni0) * 1.33) * Rdens;
  wk[I_Pigen] = dmax(dmin(Qi0 - qi, qv - qsati), 0.0) / dt;

  /* accretion, :1087-1145 */
  double Esi_mod = dmin(c->Esi, c->Esi * exp(c->gamma_sacr * temc));
  double Egs_mod = dmin(c->Egs, c->Egs * exp(c->gamma_gacs * temc));
  double Pracw_orig = qc * 0.25 * PI * c->Erw * N0r * Cr * c->GAM_3dr * RLMDr_3dr * rho_fact;
  zerosw = 0.5 - copysign(0.5, qc * qr - 1.0E-12);
  double Pracw_kk = 67.0 * exp(log(qc * qr + zerosw) * 1.15) * (1.0 - zerosw);
  wk[I_Pracw] = (1.0 - sw_kk2000) * Pracw_orig + (sw_kk2000)*Pracw_kk;
  wk[I_Psacw] = qc * 0.25 * PI * c->Esw * Cs * MOMs_2ds * rho_fact;
  wk[I_Pgacw] = qc * 0.25 * PI * c->Egw * N0g * Cg * c->GAM_3dg * RLMDg_3dg * rho_fact;
  wk[I_Praci] = qi * 0.25 * PI * c->Eri * N0r * Cr * c->GAM_3dr * RLMDr_3dr * rho_fact;
  wk[I_Psaci] = qi * 0.25 * PI * Esi_mod * Cs * MOMs_2ds * rho_fact;
  wk[I_Pgaci] = qi * 0.25 * PI * c->Egi * N0g * Cg * c->GAM_3dg * RLMDg_3dg * rho_fact;
  wk[I_Piacr] = qi * Ar / c->mi * 0.25 * PI * c->Eri * N0r * Cr * c->GAM_6dr * RLMDr_6dr * rho_fact;
  wk[I_Psacr] = Ar * 0.25 * PI * Rdens * c->Esr * N0r * fabs(Vtr - Vts) *
                (c->GAM_1br * RLMDr_1br * MOMs_2 + 2.0 * c->GAM_2br * RLMDr_2br * MOMs_1 +
                 c->GAM_3br * RLMDr_3br * MOMs_0);
  wk[I_Pgacr] = Ar * 0.25 * PI * Rdens * c->Egr * N0g * N0r * fabs(Vtg - Vtr) *
                (c->GAM_1br * RLMDr_1br * GAM_3 * RLMDg_3 + 2.0 * c->GAM_2br * RLMDr_2br * GAM_2 * RLMDg_2 +
                 c->GAM_3br * RLMDr_3br * GAM * RLMDg);
  wk[I_Pracs] = As * 0.25 * PI * Rdens * c->Esr * N0r * fabs(Vtr - Vts) *
                (MOMs_0bs * GAM_3 * RLMDr_3 + 2.0 * MOMs_1bs * GAM_2 * RLMDr_2 + MOMs_2bs * GAM * RLMDr);
  wk[I_Pgacs] = As * 0.25 * PI * Rdens * Egs_mod * N0g * fabs(Vtg - Vts) *
                (MOMs_0bs * GAM_3 * RLMDg_3 + 2.0 * MOMs_1bs * GAM_2 * RLMDg_2 + MOMs_2bs * GAM * RLMDg);

  /* autoconversion, :1147-1172 (the reference evaluates Praut_kk twice; the
   * second assignment, :1156, is the one used) */
  double rhoqc = dens * qc * 1000.0;
  double Dc = 0.146 - 5.964E-2 * log(Nc / 2000.0);
  double Praut_berry = Rdens * 1.67E-5 * rhoqc * rhoqc / (5.0 + 3.66E-2 * Nc / (Dc * rhoqc + EPS));
  double Praut_kk = c->kk_aut * pow(qc, 2.47) * pow(Nc, -1.79);
  wk[I_Praut] = (1.0 - sw_kk2000) * Praut_berry + sw_kk2000 * Praut_kk;
  double betai = dmin(c->beta_saut, c->beta_saut * exp(c->gamma_saut * temc));
  wk[I_Psaut] = dmax(betai * (qi - c->qicrt_saut), 0.0);
  double betas = dmin(c->beta_gaut, c->beta_gaut * exp(c->gamma_gaut * temc));
  wk[I_Pgaut] = dmax(betas * (qs - c->qscrt_gaut), 0.0);

  /* evaporation, sublimation, melting, freezing, :1174-1247 */
  double Ka = (Ka0 + dKa_dT * temc);
  double Kd = (Kd0 + dKd_dT * temc) * PRE00 / pre;
  double Nu = (nu0 + dnu_dT * temc) * Rdens;
  double Glv = 1.0 / (LHV0 / (Ka * temp) * (LHV0 / (Rvap * temp) - 1.0) + 1.0 / (Kd * dens * qsatl));
  double Giv = 1.0 / (LHS0 / (Ka * temp) * (LHS0 / (Rvap * temp) - 1.0) + 1.0 / (Kd * dens * qsati));
  double Gil = 1.0 / (LHF0 / (Ka * temc));
  double ventr = c->f1r * GAM_2 * RLMDr_2 + c->f2r * sqrt(Cr * rho_fact / Nu * RLMDr_5dr) * c->GAM_5dr_h;
  wk[I_Prevp] = 2.0 * PI * Rdens * N0r * (1.0 - dmin(Sliq, 1.0)) * Glv * ventr;
  double rhoqi = dmax(dens * qi, EPS);
  double XNi = dmin(dmax(5.38E+7 * exp(log(rhoqi) * 0.75), 1.0E+3), 1.0E+6);
  double XMi = rhoqi / XNi;
  double Di = dmin(c->Di_a * sqrt(XMi), c->Di_max);
  double tmp = 4.0 * Di * XNi * Rdens * (Sice - 1.0) * Giv;
  wk[I_Pidep] = (wk[I_spsati]) * (tmp);
  wk[I_Pisub] = (1.0 - wk[I_spsati]) * (-tmp);
  double sw = (0.5 - copysign(0.5, temc + 40.0));
  wk[I_Pihom] = sw * qc / dt;
  sw = (0.5 + copysign(0.5, temc + 40.0)) * (0.5 - copysign(0.5, temc));
  wk[I_Pihtr] = sw * (dens / CONST_DWATR * (qc * qc) / (c->Nc_ihtr * 1.0E+6)) * c->B_frz *
                (exp(-c->A_frz * temc) - 1.0);
  sw = (0.5 + copysign(0.5, temc));
  wk[I_Pimlt] = sw * qi / dt;
  double vents = c->f1s * MOMs_1 + c->f2s * sqrt(Cs * rho_fact / Nu) * MOMs_5ds_h;
  tmp = 2.0 * PI * Rdens * (Sice - 1.0) * Giv * vents;
  wk[I_Psdep] = (wk[I_spsati]) * (tmp);
  wk[I_Pssub] = (1.0 - wk[I_spsati]) * (-tmp);
  wk[I_Psmlt] = 2.0 * PI * Rdens * Gil * vents + CONST_CL * temc / LHF0 * (wk[I_Psacw] + wk[I_Psacr]);
  wk[I_Psmlt] = dmax(wk[I_Psmlt], 0.0);
  double ventg = c->f1g * GAM_2 * RLMDg_2 + c->f2g * sqrt(Cg * rho_fact / Nu * RLMDg_5dg) * c->GAM_5dg_h;
  tmp = 2.0 * PI * Rdens * N0g * (Sice - 1.0) * Giv * ventg;
  wk[I_Pgdep] = (wk[I_spsati]) * (tmp);
  wk[I_Pgsub] = (1.0 - wk[I_spsati]) * (-tmp);
  wk[I_Pgmlt] = 2.0 * PI * Rdens * N0g * Gil * ventg + CONST_CL * temc / LHF0 * (wk[I_Pgacw] + wk[I_Pgacr]);
  wk[I_Pgmlt] = dmax(wk[I_Pgmlt], 0.0);
  wk[I_Pgfrz] = 2.0 * PI * Rdens * N0r * 60.0 * c->B_frz * Ar * (exp(-c->A_frz * temc) - 1.0) * RLMDr_7;
  double dt1 = (exp(log(c->mi50) * ma2) - exp(log(c->mi40) * ma2)) / (a1 * ma2);
  double Ni50 = qi * dt / (c->mi50 * dt1);
  wk[I_Psfw] = Ni50 * (a1 * pow(c->mi50, a2) + PI * c->Eiw * dens * qc * c->Ri50 * c->Ri50 * c->vti50);
  wk[I_Psfi] = qi / dt1;

  /* limiters, :1249-1296 */
  NSW6O_SITE(SITE_LIMITER);
  wk[I_Pigen] = dmin(wk[I_Pigen], wk[I_dqv_dt]) * (wk[I_iceflg]) * sw_expice;
  wk[I_Pidep] = dmin(wk[I_Pidep], wk[I_dqv_dt]) * (wk[I_iceflg]) * sw_expice;
  wk[I_Psdep] = dmin(wk[I_Psdep], wk[I_dqv_dt]) * (wk[I_iceflg]);
  wk[I_Pgdep] = dmin(wk[I_Pgdep], wk[I_dqv_dt]) * (wk[I_iceflg]);
  wk[I_Pracw] = wk[I_Pracw] + wk[I_Psacw] * (1.0 - wk[I_iceflg]) + wk[I_Pgacw] * (1.0 - wk[I_iceflg]);
  wk[I_Praut] = dmin(wk[I_Praut], wk[I_dqc_dt]);
  wk[I_Pracw] = dmin(wk[I_Pracw], wk[I_dqc_dt]);
  wk[I_Pihom] = dmin(wk[I_Pihom], wk[I_dqc_dt]) * (wk[I_iceflg]) * sw_expice;
  wk[I_Pihtr] = dmin(wk[I_Pihtr], wk[I_dqc_dt]) * (wk[I_iceflg]) * sw_expice;
  wk[I_Psacw] = dmin(wk[I_Psacw], wk[I_dqc_dt]) * (wk[I_iceflg]);
  wk[I_Psfw] = dmin(wk[I_Psfw], wk[I_dqc_dt]) * (wk[I_iceflg]) * sw_bergeron;
  wk[I_Pgacw] = dmin(wk[I_Pgacw], wk[I_dqc_dt]) * (wk[I_iceflg]);
  wk[I_Prevp] = dmin(wk[I_Prevp], wk[I_dqr_dt]);
  wk[I_Piacr] = dmin(wk[I_Piacr], wk[I_dqr_dt]) * (wk[I_iceflg]);
  wk[I_Psacr] = dmin(wk[I_Psacr], wk[I_dqr_dt]) * (wk[I_iceflg]);
  wk[I_Pgacr] = dmin(wk[I_Pgacr], wk[I_dqr_dt]) * (wk[I_iceflg]);
  wk[I_Pgfrz] = dmin(wk[I_Pgfrz], wk[I_dqr_dt]) * (wk[I_iceflg]);
  wk[I_Pisub] = dmin(wk[I_Pisub], wk[I_dqi_dt]) * (wk[I_iceflg]) * sw_expice;
  wk[I_Pimlt] = dmin(wk[I_Pimlt], wk[I_dqi_dt]) * (1.0 - wk[I_iceflg]) * sw_expice;
  wk[I_Psaut] = dmin(wk[I_Psaut], wk[I_dqi_dt]) * (wk[I_iceflg]);
  wk[I_Praci] = dmin(wk[I_Praci], wk[I_dqi_dt]) * (wk[I_iceflg]);
  wk[I_Psaci] = dmin(wk[I_Psaci], wk[I_dqi_dt]) * (wk[I_iceflg]);
  wk[I_Psfi] = dmin(wk[I_Psfi], wk[I_dqi_dt]) * (wk[I_iceflg]) * sw_bergeron;
  wk[I_Pgaci] = dmin(wk[I_Pgaci], wk[I_dqi_dt]) * (wk[I_iceflg]);
  wk[I_Pssub] = dmin(wk[I_Pssub], wk[I_dqs_dt]) * (wk[I_iceflg]);
  wk[I_Psmlt] = dmin(wk[I_Psmlt], wk[I_dqs_dt]) * (1.0 - wk[I_iceflg]);
  wk[I_Pgaut] = dmin(wk[I_Pgaut], wk[I_dqs_dt]) * (wk[I_iceflg]);
  wk[I_Pracs] = dmin(wk[I_Pracs], wk[I_dqs_dt]) * (wk[I_iceflg]);
  wk[I_Pgacs] = dmin(wk[I_Pgacs], wk[I_dqs_dt]);
  wk[I_Pgsub] = dmin(wk[I_Pgsub], wk[I_dqg_dt]) * (wk[I_iceflg]);
  wk[I_Pgmlt] = dmin(wk[I_Pgmlt], wk[I_dqg_dt]) * (1.0 - wk[I_iceflg]);
  wk[I_Piacr_s] = (1.0 - wk[I_delta1]) * wk[I_Piacr];
  wk[I_Piacr_g] = (wk[I_delta1]) * wk[I_Piacr];
  wk[I_Praci_s] = (1.0 - wk[I_delta1]) * wk[I_Praci];
  wk[I_Praci_g] = (wk[I_delta1]) * wk[I_Praci];
  wk[I_Psacr_s] = (wk[I_delta2]) * wk[I_Psacr];
  wk[I_Psacr_g] = (1.0 - wk[I_delta2]) * wk[I_Psacr];
  wk[I_Pracs] = (1.0 - wk[I_delta2]) * wk[I_Pracs];

  double net, fac, fac_sw;
  /* [QC] loss limiter, :1298-1320 */
  net = +wk[I_Pimlt] - wk[I_Praut] - wk[I_Pracw] - wk[I_Pihom] - wk[I_Pihtr] - wk[I_Psacw] - wk[I_Psfw] -
        wk[I_Pgacw];
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-wk[I_dqc_dt] / (net - fac_sw), 1.0);
  wk[I_Pimlt] = wk[I_Pimlt] * fac;
  wk[I_Praut] = wk[I_Praut] * fac;
  wk[I_Pracw] = wk[I_Pracw] * fac;
  wk[I_Pihom] = wk[I_Pihom] * fac;
  wk[I_Pihtr] = wk[I_Pihtr] * fac;
  wk[I_Psacw] = wk[I_Psacw] * fac;
  wk[I_Psfw] = wk[I_Psfw] * fac;
  wk[I_Pgacw] = wk[I_Pgacw] * fac;
  /* [QI] :1322-1354 */
  net = +wk[I_Pigen] + wk[I_Pidep] + wk[I_Pihom] + wk[I_Pihtr] - wk[I_Pisub] - wk[I_Pimlt] - wk[I_Psaut] -
        wk[I_Praci_s] - wk[I_Psaci] - wk[I_Psfi] - wk[I_Praci_g] - wk[I_Pgaci];
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-wk[I_dqi_dt] / (net - fac_sw), 1.0);
  wk[I_Pigen] = wk[I_Pigen] * fac;
  wk[I_Pidep] = wk[I_Pidep] * fac;
  wk[I_Pihom] = wk[I_Pihom] * fac;
  wk[I_Pihtr] = wk[I_Pihtr] * fac;
  wk[I_Pisub] = wk[I_Pisub] * fac;
  wk[I_Pimlt] = wk[I_Pimlt] * fac;
  wk[I_Psaut] = wk[I_Psaut] * fac;
  wk[I_Praci_s] = wk[I_Praci_s] * fac;
  wk[I_Psaci] = wk[I_Psaci] * fac;
  wk[I_Psfi] = wk[I_Psfi] * fac;
  wk[I_Praci_g] = wk[I_Praci_g] * fac;
  wk[I_Pgaci] = wk[I_Pgaci] * fac;
  /* [QR] :1357-1385 */
  net = +wk[I_Praut] + wk[I_Pracw] + wk[I_Psmlt] + wk[I_Pgmlt] - wk[I_Prevp] - wk[I_Piacr_s] -
        wk[I_Psacr_s] - wk[I_Piacr_g] - wk[I_Psacr_g] - wk[I_Pgacr] - wk[I_Pgfrz];
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-wk[I_dqr_dt] / (net - fac_sw), 1.0);
  wk[I_Praut] = wk[I_Praut] * fac;
  wk[I_Pracw] = wk[I_Pracw] * fac;
  wk[I_Psmlt] = wk[I_Psmlt] * fac;
  wk[I_Pgmlt] = wk[I_Pgmlt] * fac;
  wk[I_Prevp] = wk[I_Prevp] * fac;
  wk[I_Piacr_s] = wk[I_Piacr_s] * fac;
  wk[I_Psacr_s] = wk[I_Psacr_s] * fac;
  wk[I_Piacr_g] = wk[I_Piacr_g] * fac;
  wk[I_Psacr_g] = wk[I_Psacr_g] * fac;
  wk[I_Pgacr] = wk[I_Pgacr] * fac;
  wk[I_Pgfrz] = wk[I_Pgfrz] * fac;
  /* [QV] :1387-1407 */
  net = +wk[I_Prevp] + wk[I_Pisub] + wk[I_Pssub] + wk[I_Pgsub] - wk[I_Pigen] - wk[I_Pidep] - wk[I_Psdep] -
        wk[I_Pgdep];
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-wk[I_dqv_dt] / (net - fac_sw), 1.0);
  wk[I_Prevp] = wk[I_Prevp] * fac;
  wk[I_Pisub] = wk[I_Pisub] * fac;
  wk[I_Pssub] = wk[I_Pssub] * fac;
  wk[I_Pgsub] = wk[I_Pgsub] * fac;
  wk[I_Pigen] = wk[I_Pigen] * fac;
  wk[I_Pidep] = wk[I_Pidep] * fac;
  wk[I_Psdep] = wk[I_Psdep] * fac;
  wk[I_Pgdep] = wk[I_Pgdep] * fac;
  /* [QS] :1409-1443 */
  net = +wk[I_Psdep] + wk[I_Psacw] + wk[I_Psfw] + wk[I_Piacr_s] + wk[I_Psacr_s] + wk[I_Psaut] +
        wk[I_Praci_s] + wk[I_Psaci] + wk[I_Psfi] - wk[I_Pssub] - wk[I_Psmlt] - wk[I_Pgaut] - wk[I_Pracs] -
        wk[I_Pgacs];
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-wk[I_dqs_dt] / (net - fac_sw), 1.0);
  wk[I_Psdep] = wk[I_Psdep] * fac;
  wk[I_Psacw] = wk[I_Psacw] * fac;
  wk[I_Psfw] = wk[I_Psfw] * fac;
  wk[I_Piacr_s] = wk[I_Piacr_s] * fac;
  wk[I_Psacr_s] = wk[I_Psacr_s] * fac;
  wk[I_Psaut] = wk[I_Psaut] * fac;
  wk[I_Praci_s] = wk[I_Praci_s] * fac;
  wk[I_Psaci] = wk[I_Psaci] * fac;
  wk[I_Psfi] = wk[I_Psfi] * fac;
  wk[I_Pssub] = wk[I_Pssub] * fac;
  wk[I_Psmlt] = wk[I_Psmlt] * fac;
  wk[I_Pgaut] = wk[I_Pgaut] * fac;
  wk[I_Pracs] = wk[I_Pracs] * fac;
  wk[I_Pgacs] = wk[I_Pgacs] * fac;
  /* [QG] :1445-1477 */
  net = +wk[I_Pgdep] + wk[I_Pgacw] + wk[I_Piacr_g] + wk[I_Psacr_g] + wk[I_Pgacr] + wk[I_Pgfrz] +
        wk[I_Praci_g] + wk[I_Pgaci] + wk[I_Pgaut] + wk[I_Pracs] + wk[I_Pgacs] - wk[I_Pgsub] - wk[I_Pgmlt];
  fac_sw = 0.5 + copysign(0.5, net + EPS);
  fac = fac_sw + (1.0 - fac_sw) * dmin(-wk[I_dqg_dt] / (net - fac_sw), 1.0);
  wk[I_Pgdep] = wk[I_Pgdep] * fac;
  wk[I_Pgacw] = wk[I_Pgacw] * fac;
  wk[I_Piacr_g] = wk[I_Piacr_g] * fac;
  wk[I_Psacr_g] = wk[I_Psacr_g] * fac;
  wk[I_Pgacr] = wk[I_Pgacr] * fac;
  wk[I_Pgfrz] = wk[I_Pgfrz] * fac;
  wk[I_Praci_g] = wk[I_Praci_g] * fac;
  wk[I_Pgaci] = wk[I_Pgaci] * fac;
  wk[I_Pgaut] = wk[I_Pgaut] * fac;
  wk[I_Pracs] = wk[I_Pracs] * fac;
  wk[I_Pgacs] = wk[I_Pgacs] * fac;
  wk[I_Pgsub] = wk[I_Pgsub] * fac;
  wk[I_Pgmlt] = wk[I_Pgmlt] * fac;

  /* tendencies, :1479-1559 */
  double qc_t = +wk[I_Pimlt] - wk[I_Praut] - wk[I_Pracw] - wk[I_Pihom] - wk[I_Pihtr] - wk[I_Psacw] -
                wk[I_Psfw] - wk[I_Pgacw];
  double qr_t = +wk[I_Praut] + wk[I_Pracw] + wk[I_Psmlt] + wk[I_Pgmlt] - wk[I_Prevp] - wk[I_Piacr_s] -
                wk[I_Psacr_s] - wk[I_Piacr_g] - wk[I_Psacr_g] - wk[I_Pgacr] - wk[I_Pgfrz];
  double qi_t = +wk[I_Pigen] + wk[I_Pidep] + wk[I_Pihom] + wk[I_Pihtr] - wk[I_Pisub] - wk[I_Pimlt] -
                wk[I_Psaut] - wk[I_Praci_s] - wk[I_Psaci] - wk[I_Psfi] - wk[I_Praci_g] - wk[I_Pgaci];
  double qs_t = +wk[I_Psdep] + wk[I_Psacw] + wk[I_Psfw] + wk[I_Piacr_s] + wk[I_Psacr_s] + wk[I_Psaut] +
                wk[I_Praci_s] + wk[I_Psaci] + wk[I_Psfi] - wk[I_Pssub] - wk[I_Psmlt] - wk[I_Pgaut] -
                wk[I_Pracs] - wk[I_Pgacs];
  double qg_t = +wk[I_Pgdep] + wk[I_Pgacw] + wk[I_Piacr_g] + wk[I_Psacr_g] + wk[I_Pgacr] + wk[I_Pgfrz] +
                wk[I_Praci_g] + wk[I_Pgaci] + wk[I_Pgaut] + wk[I_Pracs] + wk[I_Pgacs] - wk[I_Pgsub] -
                wk[I_Pgmlt];
  qc_t = dmax(qc_t, -wk[I_dqc_dt]);
  qr_t = dmax(qr_t, -wk[I_dqr_dt]);
  qi_t = dmax(qi_t, -wk[I_dqi_dt]);
  qs_t = dmax(qs_t, -wk[I_dqs_dt]);
  qg_t = dmax(qg_t, -wk[I_dqg_dt]);
  double qv_t = -(qc_t + qr_t + qi_t + qs_t + qg_t);
  o->drhogq[0] = rhog * qv_t * dt;
  o->drhogq[1] = rhog * qc_t * dt;
  o->drhogq[2] = rhog * qr_t * dt;
  o->drhogq[3] = rhog * qi_t * dt;
  o->drhogq[4] = rhog * qs_t * dt;
  o->drhogq[5] = rhog * qg_t * dt;
  o->Vt[0] = Vtr;
  o->Vt[1] = Vti;
  o->Vt[2] = Vts;
  o->Vt[3] = Vtg;

  /* effective radius and cloud top, :1566-1592 */
  NSW6O_SITE(SITE_DIAG);
  double xf_qc = rhoqc / Nc * 1.0E-9;
  double rf_qc = pow((c->coef_xf * xf_qc + EPS), 0.33333333);
  double r2_qc = c->coef_dgam * (rf_qc * rf_qc) * (Nc * 1.0E+6);
  double r2_qr = 0.25 * N0r * GAM_3 * RLMDr_3;
  double r3_qc = c->coef_xf * dens * qc;
  double r3_qr = c->coef_xf * dens * qr;
  zerosw = 0.5 - copysign(0.5, (r2_qc + r2_qr) - r2_min);
  o->rceff = (r3_qc + r3_qr) / (r2_qc + r2_qr + zerosw) * (1.0 - zerosw);
  sw = (0.5 + copysign(0.5, (qc + qr) - q_min)) * zerosw;
  o->rctop = (sw)*o->rceff + (1.0 - sw) * UNDEF;
  o->tctop = (sw)*temp + (1.0 - sw) * UNDEF;
  zerosw = 0.5 - copysign(0.5, r2_qc - r2_min);
  o->rceff_cld = r3_qc / (r2_qc + zerosw) * (1.0 - zerosw);
  sw = (0.5 + copysign(0.5, qc - q_min)) * zerosw;
  o->rctop_cld = (sw)*o->rceff_cld + (1.0 - sw) * UNDEF;
  o->tctop_cld = (sw)*temp + (1.0 - sw) * UNDEF;
}

/* cnvvar_rhogkin_in, mod_debug.cpp:269-330. */
static void cnvvar_rhogkin_in(const dims_t* D, const double* rhog, const double* rhogvx, const double* rhogvy,
                              const double* rhogvz, const double* rhogw, const double* C2W,
                              const double* W2C, double* rhogkin, double* rhogkin_h, double* rhogkin_v) {
  const int G = D->G, kmin = D->kmin, kmax = D->kmax;
  const size_t N = D->N;
  OMP_FOR
  for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i)
    rhogkin_h[i] = 0.5 * (rhogvx[i] * rhogvx[i] + rhogvy[i] * rhogvy[i] + rhogvz[i] * rhogvz[i]) / rhog[i];
  for (int g = 0; g < G; ++g) {
    rhogkin_h[IX(kmin - 1, g)] = 0.0;
    rhogkin_h[IX(kmax + 1, g)] = 0.0;
  }
  OMP_FOR
  for (size_t i = IX(kmin + 1, 0); i < IX(kmax + 1, 0); ++i)
    rhogkin_v[i] = 0.5 * (rhogw[i] * rhogw[i]) / (C2W[i] * rhog[i] + C2W[N + i] * rhog[i - G]);
  for (int g = 0; g < G; ++g) {
    rhogkin_v[IX(kmin - 1, g)] = 0.0;
    rhogkin_v[IX(kmin, g)] = 0.0;
    rhogkin_v[IX(kmax + 1, g)] = 0.0;
  }
  OMP_FOR
  for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i)
    rhogkin[i] = rhogkin_h[i] + (W2C[i] * rhogkin_v[i + G] + W2C[N + i] * rhogkin_v[i]);
  for (int g = 0; g < G; ++g) {
    rhogkin[IX(kmin - 1, g)] = 0.0;
    rhogkin[IX(kmax + 1, g)] = 0.0;
  }
}

/* vadv1d_prep, mod_vadv1d.cpp:231-391.  zdis is updated in place for
 * k in [mkmin-1, mkmax+1] (other levels keep their previous content). */
static void vadv1d_prep(const dims_t* D, int mkmin, int mkmax, const double* dz, const double* zh,
                        const double* wp, double* zdis, int* kcell, int* kcell_max, int* kcell_min, double dt,
                        double* wh) {
  const int G = D->G, K = D->K;
  NSW6O_PHASE(3);
  NSW6O_SITE(SITE_DEPARTURE);
  const double dt2 = pow(dt, 2);
  const double dt3 = pow(dt, 3);
  memset(wh, 0, sizeof(double) * D->N);
  for (int k = mkmin + 1; k <= mkmax; ++k)
    for (int g = 0; g < G; ++g) wh[IX(k, g)] = 0.5 * (wp[IX(k - 1, g)] + wp[IX(k, g)]);
  for (int g = 0; g < G; ++g) {
    wh[IX(mkmin, g)] = wp[IX(mkmin, g)];
    wh[IX(mkmin - 1, g)] = wp[IX(mkmin - 1, g)];
    wh[IX(mkmax + 1, g)] = wp[IX(mkmax, g)];
  }
  for (int k = mkmin + 1; k <= mkmax; ++k) {
    OMP_FOR
    for (int g = 0; g < G; ++g) {
      const double w0 = wh[IX(k, g)], wm = wh[IX(k - 1, g)], wpp = wh[IX(k + 1, g)];
      zdis[IX(k, g)] =
          dt * w0 - dt2 * w0 * (wpp - wm) / (dz[k - 1] + dz[k]) / 2.0 +
          dt3 * w0 *
              (pow((wpp - wm) / (dz[k - 1] + dz[k]), 2) +
               w0 * (((wpp - w0) / dz[k] - (w0 - wm) / dz[k - 1]) / (dz[k - 1] + dz[k]) * 2.0)) /
              6.0;
    }
  }
  for (int g = 0; g < G; ++g) {
    zdis[IX(mkmin - 1, g)] = 0.0;
    zdis[IX(mkmin, g)] = dt * wh[IX(mkmin, g)] -
                         dt2 * wh[IX(mkmin, g)] * (wh[IX(mkmin + 1, g)] - wh[IX(mkmin, g)]) / dz[mkmin] / 2.0;
    zdis[IX(mkmax + 1, g)] = dt * wh[IX(mkmax + 1, g)] -
                             dt2 * wh[IX(mkmax + 1, g)] * (wh[IX(mkmax + 1, g)] - wh[IX(mkmax, g)]) / dz[mkmax] / 2.0;
  }
  NSW6O_PHASE(2);
  for (int k = 0; k < K; ++k) {
    for (int g = 0; g < G; ++g) kcell[IX(k, g)] = k;
    kcell_min[k] = k;
    kcell_max[k] = k;
  }
  /* region-wide extrema of the departure distance, :316-353 */
  for (int k = mkmin; k <= mkmax; ++k) {
    double zzmax = DBL_MIN, zzmin = DBL_MIN;
    for (int g = 0; g < G; ++g) {
      double val = zdis[IX(k, g)];
      zzmax = val > zzmax ? val : zzmax;
      zzmin = val < zzmin ? val : zzmin;
    }
    if (zzmax > 0.0) {
      for (int k2 = k; k2 >= mkmin; --k2) {
        if ((zh[k2] <= zh[k] - zzmax) && (zh[k2 + 1] > zh[k] - zzmax)) {
          kcell_min[k] = k2;
          break;
        }
      }
    }
    if (zzmin < 0.0) {
      for (int k2 = k; k2 <= mkmax; ++k2) {
        if ((zh[k2] <= zh[k] - zzmin) && (zh[k2 + 1] > zh[k] - zzmin)) {
          kcell_max[k] = k2;
          break;
        }
      }
    }
  }
  /* per-cell departure cell, :355-384 */
  for (int k = mkmin; k <= mkmax; ++k) {
    OMP_FOR
    for (int g = 0; g < G; ++g) {
      if (kcell_min[k] == k && kcell_max[k] == k) {
        kcell[IX(k, g)] = k;
      } else {
        int kc = 0;
        for (int k2 = kcell_min[k]; k2 <= kcell_max[k]; ++k2) {
          double dep = zh[k] - zdis[IX(k, g)];
          int tmp = (int)((double)k2 * copysign(1.0, dep - zh[k2]) * copysign(1.0, zh[k2 + 1] - dep));
          kc = kc > tmp ? kc : tmp;
        }
        kcell[IX(k, g)] = kc;
      }
    }
  }
  for (size_t i = 0; i < D->N; ++i) {
    if (kcell[i] == 0) kcell[i] = mkmin;
    if (kcell[i] == mkmax + 1) kcell[i] = mkmax;
  }
  NSW6O_SITE(SITE_OTHER);
}

/* vadv1d_getflux_new, mod_vadv1d.cpp:393-450.
 *
 * In the reference's Kokkos lambda the level index k is a size_t
 * (mod_vadv1d.cpp:415), so f2 = (k-1) - k2 and f3 = k2 - k (:420-421) are
 * evaluated in unsigned arithmetic and are never negative: their
 * copysign(1, f) + 1 factors are always 2.  The effective weight is therefore
 * fact = +dz(k2) for k2 > kcell, -dz(k2) for k2 < kcell and 0 at kcell.  The
 * restatement reproduces that arithmetic. */
static void vadv1d_getflux(const dims_t* D, int mkmin, int mkmax, const double* dz, const double* rhof,
                           const double* zdis0, const int* kcell, const int* kcell_max, const int* kcell_min,
                           double* frhof) {
  const int G = D->G;
  NSW6O_SITE(SITE_FLUXSUM);
  memset(frhof, 0, sizeof(double) * D->N);
  for (int k = mkmin; k <= mkmax; ++k) {
    OMP_FOR
    for (int g = 0; g < G; ++g) {
      const size_t i = IX(k, g);
      const int kc = kcell[i];
      double zdis = 0.0, f = 0.0;
      if (kcell_min[k] == k && kcell_max[k] == k) {
        zdis = zdis0[i];
      } else {
        for (int k2 = kcell_min[k]; k2 <= kcell_max[k]; ++k2) {
          const size_t ku = (size_t)k, k2u = (size_t)k2;
          double f1 = (double)(k2 - (kc + 1));
          double f2 = (double)((ku - 1) - k2u);
          double f3 = (double)(k2u - ku);
          double f4 = (double)((kc - 1) - k2);
          double fact = dz[k2] * 0.25 *
                        ((copysign(1.0, f1) + 1.0) * (copysign(1.0, f2) + 1.0) -
                         (copysign(1.0, f3) + 1.0) * (copysign(1.0, f4) + 1.0));
          f = f + rhof[IX(k2, g)] * fact;
          zdis = zdis0[i] - fact;
        }
      }
      f = f + rhof[IX(kc, g)] * zdis;
      frhof[i] = f;
    }
  }
  NSW6O_SITE(SITE_EPSFILTER);
  OMP_FOR
  for (size_t i = 0; i < D->N; ++i) frhof[i] = frhof[i] * (0.5 + copysign(0.5, fabs(frhof[i]) - CONST_EPS));
  NSW6O_SITE(SITE_OTHER);
}

/* ------------------------------------------------------------------ driver */
int nsw6o_mp_driver(int gall, int kall, const double* gz_in, const double* gzh_in, const nsw6o_params* prm,
                    double* const* a, double dt, double ct, int itelim, int* status) {
  (void)ct;
  if (gall <= 0 || kall < 5 || !a || !gz_in || !gzh_in) return 1;
  for (int i = 0; i < A_COUNT; ++i)
    if (!a[i]) return 1;
  if (status) status[0] = status[1] = status[2] = status[3] = 0;
  if (itelim <= 0) itelim = 100;

  nsw6o_params pdef;
  if (!prm) {
    nsw6o_default_params(&pdef);
    prm = &pdef;
  }
  consts_t C;
  make_consts(&C, prm);
  dims_t DD = {gall, kall, 1, kall - 2, (size_t)gall * (size_t)kall};
  const dims_t* D = &DD;
  const int G = gall, K = kall, kmin = 1, kmax = kall - 2;
  const size_t N = D->N;
  double* gmem = zalloc(11 * (size_t)K);
  grid_t GR;
  make_grid(&GR, K, gz_in, gzh_in, gmem);

  double *rhog = a[A_rhog], *rhogvx = a[A_rhogvx], *rhogvy = a[A_rhogvy], *rhogvz = a[A_rhogvz];
  double *rhogw = a[A_rhogw], *rhoge = a[A_rhoge], *rhogq = a[A_rhogq];
  const double *vx = a[A_vx], *vy = a[A_vy], *vz = a[A_vz];
  double *rho = a[A_rho], *tem = a[A_tem], *pre = a[A_pre], *q = a[A_q], *qd = a[A_qd];
  double *precip = a[A_precip], *iso1 = a[A_ISO1], *iso2 = a[A_ISO2];
  double *precip_rhoe = a[A_precip_rhoe], *precip_lh_heat = a[A_precip_lh_heat];
  double *precip_rhophi = a[A_precip_rhophi], *precip_rhokin = a[A_precip_rhokin];
  double *rceff = a[A_re_liquid], *re_solid = a[A_re_solid], *rceff_cld = a[A_re_cld];
  double *rctop = a[A_rctop], *rwtop = a[A_rwtop], *tctop = a[A_tctop];
  const double *gsgam2 = a[A_gsgam2], *gsgam2h = a[A_gsgam2h], *gam2 = a[A_gam2], *gam2h = a[A_gam2h];
  const double *ix = a[A_ix], *iy = a[A_iy], *iz = a[A_iz], *jx = a[A_jx], *jy = a[A_jy], *jz = a[A_jz];
  const double* z = a[A_z];
  double *GDCLW = a[A_GDCLW], *GDCFRC = a[A_GDCFRC], *frain = a[A_GPREC];

  /* work arrays (all zero-initialised, as the reference's Views are) */
  double* drhogq = zalloc(6 * N);
  double *psatl = zalloc(N), *qsatl = zalloc(N), *psati = zalloc(N), *qsati = zalloc(N), *Nc = zalloc(N);
  double *a1 = zalloc(N), *a2 = zalloc(N), *ma2 = zalloc(N);
  double* Vt = zalloc(6 * N);
  double *cva = zalloc(N), *rgs = zalloc(N), *rgsh = zalloc(N), *qdw = zalloc(N), *cvw = zalloc(N);
  double *rctop_cld = zalloc(G), *tctop_cld = zalloc(G);

  /* mp_driver: zero the outputs, mod_mp_driver.cpp:464-488 */
  for (int g = 0; g < 2 * G; ++g) precip[g] = iso1[g] = iso2[g] = 0.0;
  for (size_t i = 0; i < N; ++i) GDCLW[i] = GDCFRC[i] = frain[i] = 0.0;
  for (int g = 0; g < G; ++g) precip_rhoe[g] = precip_lh_heat[g] = precip_rhophi[g] = precip_rhokin[g] = 0.0;

  /* ---- mp_nsw6_new::init, mod_mp_nsw6.cpp:439-518 */
  NSW6O_PHASE(1);
  negative_filter(D, rhog, rhoge, rhogq, rho, tem, pre, q, gsgam2, qdw, cvw);
  for (size_t i = 0; i < N; ++i) Nc[i] = C.Nc_def;  /* TagAerosolF, :681-684 */
  psat_fn(D, &C, tem, psatl, C.CPovR_liq, C.LovR_liq);
  psat_fn(D, &C, tem, psati, C.CPovR_ice, C.LovR_ice);
  OMP_FOR
  for (size_t i = 0; i < N; ++i) {  /* TagSATWater, :686-690 */
    qsatl[i] = psatl[i] / (rho[i] * CONST_Rvap * tem[i]);
    qsati[i] = psati[i] / (rho[i] * CONST_Rvap * tem[i]);
  }
  bergeron(D, tem, a1, a2, ma2);

  /* ---- mp_nsw6_new::compute, mod_mp_nsw6.cpp:520-674 */
  for (int k = kmin; k <= kmax; ++k) {
    OMP_FOR
    for (int g = 0; g < G; ++g) {
      const size_t i = IX(k, g);
      double qin[6];
      for (int nq = 0; nq < 6; ++nq) qin[nq] = q[nq * N + i];
      bigloop_out_t o;
      big_loop_cell(&C, rho[i], tem[i], qin, qsatl[i], qsati[i], Nc[i], a1[i], a2[i], ma2[i], pre[i], rhog[i],
                    dt, &o);
      for (int nq = 0; nq < 6; ++nq) drhogq[nq * N + i] = o.drhogq[nq];
      Vt[I_QR * N + i] = o.Vt[0];
      Vt[I_QI * N + i] = o.Vt[1];
      Vt[I_QS * N + i] = o.Vt[2];
      Vt[I_QG * N + i] = o.Vt[3];
      rceff[i] = o.rceff;
      rceff_cld[i] = o.rceff_cld;
      /* column scalars: the reference writes them from every k in parallel
       * (:1579-1592); sequential order, where k = kmax is written last, is used */
      rctop[g] = o.rctop;
      tctop[g] = o.tctop;
      rctop_cld[g] = o.rctop_cld;
      tctop_cld[g] = o.tctop_cld;
    }
  }
  NSW6O_SITE(SITE_OTHER);
  OMP_FOR
  for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i) {  /* TagUpdateRHOGQ, :692-700 */
    for (int nq = 0; nq < 6; ++nq) rhogq[nq * N + i] += drhogq[nq * N + i];
  }
  OMP_FOR
  for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i) {  /* TagUpdateRHOGE, :702-708 */
    rhoge[i] = rhoge[i] - CONST_LHV0 * drhogq[I_QV * N + i] + CONST_LHF0 * drhogq[I_QI * N + i] +
               CONST_LHF0 * drhogq[I_QS * N + i] + CONST_LHF0 * drhogq[I_QG * N + i];
  }
  for (int g = 0; g < G; ++g) {  /* TagUpdateCLD, :710-726 */
    rceff[IX(kmin - 1, g)] = 0.0;
    rceff_cld[IX(kmin - 1, g)] = 0.0;
    rceff[IX(kmax + 1, g)] = 0.0;
    rceff_cld[IX(kmax + 1, g)] = 0.0;
    double sw = (0.5 + copysign(0.5, tctop[g] - CONST_TEM00));
    rwtop[g] = (sw)*rctop[g] + (1.0 - sw) * CONST_UNDEF;
  }
  for (int nq = 0; nq < 6; ++nq)  /* TagPrecip, :728-732 */
    for (int g = 0; g < G; ++g) {
      Vt[nq * N + IX(kmin - 1, g)] = 0.0;
      Vt[nq * N + IX(kmax + 1, g)] = 0.0;
    }
  for (int nq = NQW_STR; nq <= NQW_END; ++nq) {  /* TagUpdateMassConc, :734-737 */
    OMP_FOR
    for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i) q[nq * N + i] = rhogq[nq * N + i] / rhog[i];
  }
  thrmdyn_qd(D, q, qd);
  thrmdyn_cv(D, qd, q, cva);
  OMP_FOR
  for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i) {  /* TagUpdateTEM, :739-744 */
    tem[i] = rhoge[i] / (rhog[i] * cva[i]);
    rgs[i] = gam2[i] / gsgam2[i];
    rgsh[i] = gam2h[i] / gsgam2h[i];
  }

  /* ---- precip_transport_new, mod_precip_transport.cpp:573-1087 */
  NSW6O_PHASE(2);
  NSW6O_SITE(SITE_OTHER);
  {
    double *rhogkin = zalloc(N), *rhogkin_h = zalloc(N), *rhogkin_v = zalloc(N);
    double *rhoq = zalloc(N), *rhoeq = zalloc(N), *rhophiq = zalloc(N), *rhokin_h = zalloc(N);
    double *rhokin_v = zalloc(N), *rhouq = zalloc(N), *rhovq = zalloc(N), *rhowq = zalloc(N);
    double *fprec_q = zalloc(N), *fprec_rhoe = zalloc(N), *fprec_rhophi = zalloc(N);
    double *fprec_rhokin_h = zalloc(N), *fprec_rhokin_v = zalloc(N), *fprec_rhou = zalloc(N);
    double *fprec_rhov = zalloc(N), *fprec_rhow = zalloc(N);
    double *drhoq = zalloc(6 * N), *drhoe = zalloc(N), *drhophi = zalloc(N), *drhokin_h = zalloc(N);
    double *drhokin_v = zalloc(N), *drhogu = zalloc(N), *drhogv = zalloc(N), *drhogw = zalloc(N);
    double *zdis0 = zalloc(N), *zdis0h = zalloc(N), *Vtermh = zalloc(N), *qh = zalloc(N);
    double *ein = zalloc(N), *tmp = zalloc(N), *tmp_h = zalloc(N), *tmp_v = zalloc(N), *tmp2 = zalloc(N);
    double *C2W = zalloc(2 * N), *W2C = zalloc(2 * N), *wh = zalloc(N);
    int* kcell = (int*)calloc(N, sizeof(int));
    int* kcellh = (int*)calloc(N, sizeof(int));
    int *kcell_max = (int*)calloc((size_t)K, sizeof(int)), *kcell_min = (int*)calloc((size_t)K, sizeof(int));
    int *kcellh_max = (int*)calloc((size_t)K, sizeof(int)), *kcellh_min = (int*)calloc((size_t)K, sizeof(int));

    /* metric factors, :715-737 */
    for (int k = kmin; k <= kmax + 1; ++k)
      for (int g = 0; g < G; ++g) {
        C2W[IX(k, g)] = GR.afact[k] / gsgam2[IX(k, g)] * gsgam2h[IX(k, g)];
        C2W[N + IX(k, g)] = GR.bfact[k] / gsgam2[IX(k - 1, g)] * gsgam2h[IX(k, g)];
      }
    for (int g = 0; g < G; ++g) C2W[IX(kmin - 1, g)] = C2W[N + IX(kmin - 1, g)] = 0.0;
    for (int k = kmin - 1; k <= kmax; ++k)
      for (int g = 0; g < G; ++g) {
        W2C[IX(k, g)] = GR.cfact[k] * gsgam2[IX(k, g)] / gsgam2h[IX(k + 1, g)];
        W2C[N + IX(k, g)] = GR.dfact[k] * gsgam2[IX(k, g)] / gsgam2h[IX(k + 1, g)];
      }
    for (int g = 0; g < G; ++g) W2C[IX(kmax + 1, g)] = W2C[N + IX(kmax + 1, g)] = 0.0;

    cnvvar_rhogkin_in(D, rhog, rhogvx, rhogvy, rhogvz, rhogw, C2W, W2C, rhogkin, rhogkin_h, rhogkin_v);

    for (int g = 0; g < G; ++g) {  /* :758-765 */
      precip[g] = 0.0;
      precip_rhoe[g] = 0.0;
      precip_lh_heat[g] = 0.0;
      precip_rhophi[g] = 0.0;
      precip_rhokin[g] = 0.0;
    }

    /* QR, QS, QG sediment ("3WATER", mod_mp_nsw6.cpp:583-600) */
    static const int sed[3] = {I_QR, I_QS, I_QG};
    for (int t = 0; t < 3; ++t) {
      const int nq = sed[t];
      double* Vterm = Vt + (size_t)nq * N;
      double* rhogq_n = rhogq + (size_t)nq * N;
      double* q_n = q + (size_t)nq * N;
      vadv1d_prep(D, kmin, kmax, GR.dgz, GR.gzh, Vterm, zdis0, kcell, kcell_max, kcell_min, dt, wh);
      OMP_FOR
      for (size_t i = 0; i < N; ++i) rhoq[i] = rhogq_n[i] * rgs[i];
      vadv1d_getflux(D, kmin, kmax, GR.dgz, rhoq, zdis0, kcell, kcell_max, kcell_min, fprec_q);
      for (int k = kmin; k <= kmax; ++k)
        for (int g = 0; g < G; ++g)
          drhoq[nq * N + IX(k, g)] = -(fprec_q[IX(k + 1, g)] - fprec_q[IX(k, g)]) * GR.rdgz[k];

      OMP_FOR
      for (size_t i = 0; i < N; ++i) {  /* :796-808 */
        const int g = (int)(i % (size_t)G);
        rhoeq[i] = rhogq_n[i] * rgs[i] * CONST_CVdry * tem[i];
        rhophiq[i] = rhogq_n[i] * rgs[i] * CONST_GRAV * z[i];
        rhokin_h[i] = q_n[i] * rgs[i] * rhogkin_h[i];
        rhouq[i] = rhogq_n[i] * rgs[i] * (vx[i] * ix[g] + vy[i] * iy[g] + vz[i] * iz[g]);
        rhovq[i] = rhogq_n[i] * rgs[i] * (vx[i] * jx[g] + vy[i] * jy[g] + vz[i] * jz[g]);
      }
      vadv1d_getflux(D, kmin, kmax, GR.dgz, rhoeq, zdis0, kcell, kcell_max, kcell_min, fprec_rhoe);
      vadv1d_getflux(D, kmin, kmax, GR.dgz, rhophiq, zdis0, kcell, kcell_max, kcell_min, fprec_rhophi);
      vadv1d_getflux(D, kmin, kmax, GR.dgz, rhokin_h, zdis0, kcell, kcell_max, kcell_min, fprec_rhokin_h);
      vadv1d_getflux(D, kmin, kmax, GR.dgz, rhouq, zdis0, kcell, kcell_max, kcell_min, fprec_rhou);
      vadv1d_getflux(D, kmin, kmax, GR.dgz, rhovq, zdis0, kcell, kcell_max, kcell_min, fprec_rhov);
      for (int k = kmin; k <= kmax; ++k)
        for (int g = 0; g < G; ++g) {
          const size_t i = IX(k, g), ip = IX(k + 1, g);
          const double r = GR.rdgz[k];
          drhoe[i] = drhoe[i] - (fprec_rhoe[ip] - fprec_rhoe[i]) * r;
          drhophi[i] = drhophi[i] - (fprec_rhophi[ip] - fprec_rhophi[i]) * r;
          drhokin_h[i] = drhokin_h[i] - (fprec_rhokin_h[ip] - fprec_rhokin_h[i]) * r;
          drhogu[i] = drhogu[i] - (fprec_rhou[ip] - fprec_rhou[i]) * r;
          drhogv[i] = drhogv[i] - (fprec_rhov[ip] - fprec_rhov[i]) * r;
        }

      /* half levels, :845-898 */
      for (int k = kmin + 1; k <= kmax - 1; ++k)
        for (int g = 0; g < G; ++g) Vtermh[IX(k, g)] = 0.5 * (Vterm[IX(k, g)] + Vterm[IX(k - 1, g)]);
      for (int g = 0; g < G; ++g) {
        Vtermh[IX(kmin - 1, g)] = 0.0;
        Vtermh[IX(kmin, g)] = 0.0;
        Vtermh[IX(kmax, g)] = 0.0;
        Vtermh[IX(kmax + 1, g)] = 0.0;
      }
      vadv1d_prep(D, kmin + 1, kmax, GR.dgzh, GR.gz_shift, Vtermh, zdis0h, kcellh, kcellh_max, kcellh_min, dt,
                  wh);
      for (int k = kmin + 1; k <= kmax; ++k)
        for (int g = 0; g < G; ++g) qh[IX(k, g)] = 0.5 * (q_n[IX(k, g)] + q_n[IX(k - 1, g)]) * rgsh[IX(k, g)];
      for (int g = 0; g < G; ++g) {
        qh[IX(kmin - 1, g)] = 0.0;
        qh[IX(kmin, g)] = 0.0;
        qh[IX(kmax + 1, g)] = 0.0;
      }
      for (size_t i = IX(kmin + 1, 0); i < IX(kmax + 1, 0); ++i) {
        rhokin_v[i] = qh[i] * rhogkin_v[i];
        rhowq[i] = qh[i] * rhogw[i];
      }
      /* the reference passes the full-level kcell_max here (:890, :892) */
      vadv1d_getflux(D, kmin + 1, kmax, GR.dgzh, rhokin_v, zdis0h, kcellh, kcell_max, kcellh_min, fprec_rhokin_v);
      vadv1d_getflux(D, kmin + 1, kmax, GR.dgzh, rhowq, zdis0h, kcellh, kcell_max, kcellh_min, fprec_rhow);
      for (int k = kmin + 1; k <= kmax; ++k)
        for (int g = 0; g < G; ++g) {
          const size_t i = IX(k, g), im = IX(k - 1, g);
          drhokin_v[i] = drhokin_v[i] - (fprec_rhokin_v[i] - fprec_rhokin_v[im]) * GR.rdgzh[k];
          drhogw[i] = drhogw[i] - (fprec_rhow[i] - fprec_rhow[im]) * GR.rdgzh[k];
        }

      /* precipitation on the ground, :900-954 */
      if (nq == I_QR) {
        for (int g = 0; g < G; ++g) precip[g] = precip[g] - fprec_q[IX(kmin, g)] / dt;
        for (int k = kmin; k <= kmax; ++k)
          for (int g = 0; g < G; ++g) frain[IX(k, g)] = -fprec_q[IX(k, g)] / dt;
        for (int g = 0; g < G; ++g) {
          frain[IX(kmin - 1, g)] = 0.0;
          frain[IX(kmax + 1, g)] = 0.0;
        }
      } else {
        for (int g = 0; g < G; ++g) {
          precip[G + g] = precip[G + g] - fprec_q[IX(kmin, g)] / dt;
          precip_lh_heat[g] = precip_lh_heat[g] + fprec_q[IX(kmin, g)] * CONST_LHF0 / dt;
        }
      }
      for (int g = 0; g < G; ++g) {
        precip_rhoe[g] = precip_rhoe[g] - fprec_rhoe[IX(kmin, g)] / dt;
        precip_rhophi[g] = precip_rhophi[g] - fprec_rhophi[IX(kmin, g)] / dt;
        precip_rhokin[g] = precip_rhokin[g] - fprec_rhokin_h[IX(kmin, g)] / dt - fprec_rhokin_v[IX(kmin, g)] / dt;
      }
    }

    /* apply the transport tendencies, :956-989 */
    OMP_FOR
    for (size_t i = 0; i < N; ++i) {
      const int g = (int)(i % (size_t)G);
      rhoge[i] = rhoge[i] + drhoe[i] + drhophi[i];
      rhogkin_h[i] = rhogkin_h[i] + drhokin_h[i];
      rhogkin_v[i] = rhogkin_v[i] + drhokin_v[i];
      rhogvx[i] = rhogvx[i] + drhogu[i] * ix[g] + drhogv[i] * jx[g];
      rhogvy[i] = rhogvy[i] + drhogu[i] * iy[g] + drhogv[i] * jy[g];
      rhogvz[i] = rhogvz[i] + drhogu[i] * iz[g] + drhogv[i] * jz[g];
      rhogw[i] = rhogw[i] + drhogw[i];
    }
    for (int nq = 0; nq < NQ; ++nq) {
      if (nq >= NQW_STR && nq <= NQW_END) {
        OMP_FOR
        for (size_t i = 0; i < N; ++i) {
          rhogq[nq * N + i] = rhogq[nq * N + i] + drhoq[nq * N + i];
          rhog[i] = rhog[i] + drhoq[nq * N + i];
          rhoge[i] = rhoge[i] - drhoq[nq * N + i] * CONST_GRAV * z[i];
        }
      } else {
        for (size_t i = 0; i < N; ++i) rhogq[nq * N + i] = rhogq[nq * N + i] + drhoq[nq * N + i];
      }
    }

    /* KIN2EIN energy correction, :991-1011 */
    for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i)
      tmp2[i] = rhogkin_h[i] + (W2C[i] * rhogkin_v[i + G] + W2C[N + i] * rhogkin_v[i]);
    for (int g = 0; g < G; ++g) {
      tmp2[IX(kmin - 1, g)] = 0.0;
      tmp2[IX(kmax + 1, g)] = 0.0;
    }
    cnvvar_rhogkin_in(D, rhog, rhogvx, rhogvy, rhogvz, rhogw, C2W, W2C, tmp, tmp_h, tmp_v);
    for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i) rhoge[i] = rhoge[i] + (tmp2[i] - tmp[i]);

    /* final thermodynamic state at every level, :1074-1086 */
    for (int nq = 0; nq < NQ; ++nq) {
      OMP_FOR
      for (size_t i = 0; i < N; ++i) q[nq * N + i] = rhogq[nq * N + i] / rhog[i];
    }
    OMP_FOR
    for (size_t i = 0; i < N; ++i) {
      rho[i] = rhog[i] / gsgam2[i];
      ein[i] = rhoge[i] / rhog[i];
    }
    thrmdyn_qd(D, q, qd);
    /* THRMDYN_tempre, mod_thrmdyn.cpp:137-180 */
    OMP_FOR
    for (size_t i = 0; i < N; ++i) {
      double cv = 0.0, qdl = 1.0;
      for (int nq = NQW_STR; nq <= NQW_END; ++nq) {
        cv = cv + q[nq * N + i] * CONST_CVdry;
        qdl = qdl - q[nq * N + i];
      }
      cv = cv + qdl * CONST_CVdry;
      tem[i] = ein[i] / cv;
      pre[i] = rho[i] * tem[i] * (qdl * CONST_Rdry + q[I_QV * N + i] * CONST_Rvap);
    }

    free(rhogkin); free(rhogkin_h); free(rhogkin_v); free(rhoq); free(rhoeq); free(rhophiq);
    free(rhokin_h); free(rhokin_v); free(rhouq); free(rhovq); free(rhowq); free(fprec_q);
    free(fprec_rhoe); free(fprec_rhophi); free(fprec_rhokin_h); free(fprec_rhokin_v);
    free(fprec_rhou); free(fprec_rhov); free(fprec_rhow); free(drhoq); free(drhoe); free(drhophi);
    free(drhokin_h); free(drhokin_v); free(drhogu); free(drhogv); free(drhogw); free(zdis0);
    free(zdis0h); free(Vtermh); free(qh); free(ein); free(tmp); free(tmp_h); free(tmp_v); free(tmp2);
    free(C2W); free(W2C); free(wh); free(kcell); free(kcellh); free(kcell_max); free(kcell_min);
    free(kcellh_max); free(kcellh_min);
  }

  /* ---- SATURATION_adjustment (ice_adjust = false), mod_satadjust.cpp:274-362 */
  int rc = 0;
  NSW6O_SITE(SITE_NEWTON);
  {
    double *ein_moist = zalloc(N), *qsum = zalloc(N), *CVtot = zalloc(N), *rho_l = zalloc(N), *qd_l = zalloc(N);
    for (size_t i = 0; i < N; ++i) {
      ein_moist[i] = rhoge[i] / rhog[i] + q[I_QV * N + i] * CONST_LHV0;
      qsum[i] = q[I_QV * N + i] + q[I_QC * N + i];
      q[I_QV * N + i] = qsum[i];
      q[I_QC * N + i] = 0.0;
    }
    thrmdyn_cv(D, qd, q, CVtot);
    for (size_t i = 0; i < N; ++i) {
      rho_l[i] = rhog[i] / gsgam2[i];
      tem[i] = (ein_moist[i] - q[I_QV * N + i] * CONST_LHV0) / CVtot[i];
    }
    /* satadjust_liq, mod_satadjust.cpp:771-896 */
    thrmdyn_qd(D, q, qd_l);
    const double dtemp_criteria = pow(10.0, (double)(-(15 + 1) / 2));
    int first_bad = -1;
    for (size_t i = IX(kmin, 0); i < IX(kmax + 1, 0); ++i) {
      double rtem = 1.0 / (dmax(tem[i], TEM_MIN));
      double psat = CONST_PSAT0 * (pow(tem[i] * C.RTEM00, C.CPovR_liq)) * exp(C.LovR_liq * (C.RTEM00 - rtem));
      double qsat = psat / (rho_l[i] * CONST_Rvap * tem[i]);
      if (qsum[i] - qsat > CONST_EPS) {
        int converged = 0, ite;
        for (ite = 0; ite < itelim; ++ite) {
          rtem = 1.0 / (dmax(tem[i], TEM_MIN));
          psat = CONST_PSAT0 * (pow(tem[i] * C.RTEM00, C.CPovR_liq)) * exp(C.LovR_liq * (C.RTEM00 - rtem));
          qsat = psat / (rho_l[i] * CONST_Rvap * tem[i]);
          q[I_QV * N + i] = qsat;
          q[I_QC * N + i] = qsum[i] - qsat;
          double CV = qd_l[i] * CONST_CVdry;
          for (int nq = NQW_STR; nq <= NQW_END; ++nq) CV = CV + q[nq * N + i] * CONST_CVdry;
          double Emoist_new = tem[i] * CV + q[I_QV * N + i] * CONST_LHV0;
          double dqsat_dT = (C.LovR_liq / (pow(tem[i], 2)) + C.CVovR_liq / tem[i]) * qsat;
          double dCVtot_dT = dqsat_dT * (CONST_CVdry - CONST_CVdry);
          double dEmoist_dT = tem[i] * dCVtot_dT + CV + dqsat_dT * CONST_LHV0;
          double dtemp = (Emoist_new - ein_moist[i]) / dEmoist_dT;
          tem[i] = tem[i] - dtemp;
          if (fabs(dtemp) < dtemp_criteria) {
            converged = 1;
            break;
          }
          if (tem[i] * 0.0 != 0.0) break;
        }
        if (!converged && first_bad < 0) {
          first_bad = (int)i;
          if (status) {
            status[1] = (int)(i / (size_t)G);
            status[2] = (int)(i % (size_t)G);
            status[3] = ite;
          }
        }
      }
    }
    if (first_bad >= 0) {
      rc = 2;
      if (status) status[0] = 2;
    }
    for (size_t i = 0; i < N; ++i) {
      rhogq[I_QV * N + i] = rhog[i] * q[I_QV * N + i];
      rhogq[I_QC * N + i] = rhog[i] * q[I_QC * N + i];
    }
    thrmdyn_cv(D, qd, q, CVtot);
    for (size_t i = 0; i < N; ++i) rhoge[i] = rhog[i] * tem[i] * CVtot[i];
    free(ein_moist); free(qsum); free(CVtot); free(rho_l); free(qd_l);
  }

  negative_filter(D, rhog, rhoge, rhogq, rho, tem, pre, q, gsgam2, qdw, cvw);

  NSW6O_PHASE(0);
  /* ---- mp_driver epilogue, mod_mp_driver.cpp:555-612 (MP_DIV_NUM = 1) */
  for (size_t i = 0; i < N; ++i) re_solid[i] = 20.0E-6;
  const double fraction_mp = 1.0 / (double)1;
  for (int g = 0; g < 2 * G; ++g) {
    precip[g] = (0.0 + precip[g]) * fraction_mp;
    iso1[g] = (0.0 + iso1[g]) * fraction_mp;
    iso2[g] = (0.0 + iso2[g]) * fraction_mp;
  }
  for (int g = 0; g < G; ++g) {
    precip_rhoe[g] = (0.0 + precip_rhoe[g]) * fraction_mp;
    precip_lh_heat[g] = (0.0 + precip_lh_heat[g]) * fraction_mp;
    precip_rhophi[g] = (0.0 + precip_rhophi[g]) * fraction_mp;
    precip_rhokin[g] = (0.0 + precip_rhokin[g]) * fraction_mp;
  }
  for (size_t i = 0; i < N; ++i) {
    GDCLW[i] = (0.0 + GDCLW[i]) * fraction_mp;
    GDCFRC[i] = (0.0 + GDCFRC[i]) * fraction_mp;
    frain[i] = (0.0 + frain[i]) * fraction_mp;
  }

  free(gmem); free(drhogq); free(psatl); free(qsatl); free(psati); free(qsati); free(Nc);
  free(a1); free(a2); free(ma2); free(Vt); free(cva); free(rgs); free(rgsh); free(qdw); free(cvw);
  free(rctop_cld); free(tctop_cld);
  return rc;
}
