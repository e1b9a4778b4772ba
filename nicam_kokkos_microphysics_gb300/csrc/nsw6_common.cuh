// Shared definitions of the GB300 NSW6 kernels: physical constants, the scheme
// constant block passed to every kernel, launch geometry and small helpers.
#pragma once

#include <cstdint>

#include "nsw6_fpcmp.cuh"

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace nsw6 {

// ------------------------------------------------------------------ constants
// include/problemsize.h:86-135 and private module constants.
constexpr double PI = 3.141592653589793;
constexpr double EPS = 2.220446E-16;
constexpr double UNDEF = -9.9999E+30;
constexpr double GRAV = 9.79764;
constexpr double RDRY = 287.04;
constexpr double CVDRY = 717.56;
constexpr double RVAP = 461.46;
constexpr double CL = 4218.0;
constexpr double PSAT0 = 610.7;
constexpr double LHV0 = 2501000.0;
constexpr double LHS0 = 2834000.0;
constexpr double LHF0 = 333000.0;
constexpr double PSTD = 101325.0;
constexpr double TEM00 = 273.15;
constexpr double DWATR = 1000.0;
constexpr double TEM_MIN = 10.0;   // mod_satadjust.cpp:6
constexpr double DENS00 = 1.28;    // mod_mp_nsw6.cpp:8
constexpr int NQ = 6;
constexpr int I_QV = 0, I_QC = 1, I_QR = 2, I_QI = 3, I_QS = 4, I_QG = 5;

// Tile geometry.  The cell kernel gives one CTA CELL_TG columns x all interior
// levels; the column kernel one CTA 16 (kall <= 64) or 8 columns x all levels.
constexpr int CELL_TG = 32;
constexpr int CELL_THREADS = 256;
constexpr int MAX_KALL = 160;
// Above this many levels the cell kernel with the scheme switches reads the
// grid metrics and the FastMath tables from global memory instead of staging
// them in shared memory, so that its tile fits at MAX_KALL.
constexpr int CELL_SMEM_KMAX = 128;

// Scheme constants: mp_nsw6_init (mod_mp_nsw6.cpp:276-434) with the settings it
// hard-wires, the effective-radius constants of mp_nsw6_new::init
// (mod_mp_nsw6.cpp:506-517) and SATURATION_Setup (mod_satadjust.cpp:24-47).
// Built once on the host (same libm as the oracle) and passed by value; the
// mixed-precision path gets an FP32 copy (ConstsT<float>, member by member).
template <class R>
struct ConstsT {
  R Ar, As, Ag, Cr, Cs, Cg, N0r, N0s, N0g;
  R GAM_1br, GAM_2br, GAM_3br, GAM_3dr, GAM_6dr, GAM_1brdr, GAM_5dr_h;
  R GAM_1bs, GAM_2bs, GAM_3bs, GAM_3ds, GAM_1bsds, GAM_5ds_h;
  R GAM_1bg, GAM_3dg, GAM_1bgdg, GAM_5dg_h;
  R Esi, Egs, gamma_sacr, gamma_gacs, mi;
  R beta_saut, gamma_saut, qicrt_saut;
  R A_frz, B_frz, mi40, mi50, Ri50;
  R Nc_ihtr, Di_max, Di_a, ln10;
  R coef_a[10], coef_b[10];
  R Nc_def, coef_dgam, coef_xf;
  R ice_nuc, kk_aut;
  R LovR_liq, LovR_ice, RTEM00;
  R dtemp_criteria;
  // derived products that appear verbatim in the reference expressions
  R log_mi50, log_mi40;
  R Dc_berry, pow_Nc_m179;
  // constant factors of the process rates folded on the host (nsw6_cell.cuh)
  R K_rlmdr, K_rlmdg, rAs, K_vtr, K_vts, K_vtg;
  R K_sacw, K_gacw, K_raci, K_saci, K_iacr, K_sacr, K_2gam2br, K_gacr, K_g13, K_g22, K_racs;
  R K_aut, rLHF0, K_ventr1, K_ventr2, K_revp, K_ihtr, K_vents2, K_2pi, K_clf, K_ventg1, K_ventg2;
  R K_gdep, K_gfrz, K_xf, K_r2c, K_r2r;
  R roh_a[28], roh_b[28];   // per snow moment: ln10*loga and b as cubics in tems
  R ln1000;
  R XNi_eps, Di_eps;   // ice number and diameter at the floor rhoqi = EPS (no ice)
  // Scheme switches (1 = on) and the constants only the switched branches use
  // (the kernels instantiated with OPT = true read them; nsw6_options):
  //   opt_roh     Roh and Satoh (2014) snow moments (0: the classic moments)
  //   opt_expice  explicit ice generation (0: Bergeron terms, no Pigen/Pidep/
  //               Pihom/Pihtr/Pisub/Pimlt, mixed-phase saturation adjustment)
  //   opt_kk      KK2000 warm rain (0: Berry autoconversion, orig. accretion)
  //   opt_qised   QI sediments ("4WATER")
  //   opt_kin2kin kinetic-energy correction of the transport (0: KIN2EIN)
  //   opt_indir   cloud number from the CCN input (aerosol indirect effect)
  R opt_roh, opt_expice, opt_kk, opt_qised, opt_kin2kin, opt_indir;
  R Egi, K_gaci, K_gacs;                         // graupel-ice / graupel-snow accretion
  R K_rlmds, K_m0, K_m1, K_m2, K_m0bs, K_m1bs, K_m2bs, K_m2ds, K_m5dsh, K_rmomvt;   // classic snow moments
  R berg_a1[32], berg_a2[32];                    // Bergeron_param tables
  R K_berg_w;                                    // PI Eiw Ri50^2 vti50
  R sat_ulimit, sat_llimit;                      // SATURATION_Setrange of the mixed-phase adjustment
};
using Consts = ConstsT<double>;
using ConstsF = ConstsT<float>;
static_assert(sizeof(Consts) == 2 * sizeof(ConstsF), "ConstsT must hold scalars only");

// Member-by-member FP32 copy of the scheme constants (both layouts are plain
// arrays of their scalar type in the same order).
inline ConstsF consts_to_float(const Consts& c) {
  ConstsF f;
  const double* src = reinterpret_cast<const double*>(&c);
  float* dst = reinterpret_cast<float*>(&f);
  for (size_t i = 0; i < sizeof(Consts) / sizeof(double); ++i) dst[i] = (float)src[i];
  return f;
}

// Per-level grid metrics (GRD_Setup, mod_debug.cpp:92-187), device copy laid
// out as [field][kall].
enum GridField {
  GF_GZ, GF_GZH, GF_DGZ, GF_DGZH, GF_RDGZ, GF_RDGZH, GF_AFACT, GF_BFACT, GF_CFACT, GF_DFACT, GF_GZSHIFT,
  GF_RDZS, GF_RDZSH,   // 1 / (dgz(k-1) + dgz(k)) and 1 / (dgzh(k-1) + dgzh(k)), k >= 1
  GF_COUNT
};

// Argument positions of mp_driver (mod_mp_driver.h:71-124).
enum Arg {
  A_rhog, A_rhogvx, A_rhogvy, A_rhogvz, A_rhogw, A_rhoge, A_rhogq, A_vx, A_vy, A_vz, A_w,
  A_unccn, A_rho, A_tem, A_pre, A_q, A_qd, A_precip, A_ISO1, A_ISO2, A_precip_rhoe,
  A_precip_lh_heat, A_precip_rhophi, A_precip_rhokin, A_re_liquid, A_re_solid, A_re_cld,
  A_rctop, A_rwtop, A_tctop, A_frhoge_af, A_frhogqv_af, A_frhoge_rad, A_rhogqke, A_gsgam2,
  A_gsgam2h, A_gam2, A_gam2h, A_ix, A_iy, A_iz, A_jx, A_jy, A_jz, A_z, A_zh, A_GDCLW,
  A_GDCFRC, A_GPREC, A_CBMFX, A_COUNT
};

// Device status word: first failure wins.
struct DevStatus {
  int code;   // 0 ok, NSW6_ERR_NOCONV, NSW6_ERR_NAN
  int k, g, l, iters;
};

// Quotient of a 32-bit unsigned n by a divisor d >= 1 fixed for a launch,
// by a multiplication (Granlund and Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994, Theorem 4.2): with
// s = ceil(log2 d) and M = floor(2^(32+s) / d) + 1, 2^(32+s) < M d <=
// 2^(32+s) + 2^s, so floor(n M / 2^(32+s)) = floor(n / d) for every n < 2^32.
// M has 33 bits: m = M - 2^32 is kept and n M / 2^32 = umulhi(n, m) + n.
// (A 64-bit division is a long instruction sequence with conversions, which
// the FP64-bound kernels pay for.)
struct FastDiv {
  unsigned d, m, s;
  __host__ __device__ static FastDiv make(unsigned d) {
    FastDiv f{d, 0u, 0u};
    while ((1ull << f.s) < d) ++f.s;
    f.m = (unsigned)(((1ull << 32) * ((1ull << f.s) - d)) / d + 1ull);
    return f;
  }
  __host__ __device__ __forceinline__ unsigned div(unsigned n) const {
#ifdef __CUDA_ARCH__
    const unsigned long long hi = __umulhi(n, m);
#else
    const unsigned long long hi = ((unsigned long long)n * m) >> 32;
#endif
    return (unsigned)((hi + n) >> s);
  }
};

// Problem description handed to the kernels.  Array pointers follow the
// all-regions layout; per-region calls use lall = 1.
struct Problem {
  int gall, kall, kmin, kmax, lall;
  double dt, dt2, dt3;   // dt, pow(dt,2), pow(dt,3) as vadv1d_prep forms them (mod_vadv1d.cpp:265-266)
  double hdt2, sdt3;     // dt^2 / 2 and dt^3 / 6
  double rdt;            // 1 / dt
  int itelim;
  int math_lib;                // 0 table-driven transcendentals, 1 CUDA libm
  int mixed;                   // 0 plain FP64 step, 1 mixed precision (FP32 process rates)
  int opt;                     // 1: the kernels with the scheme switches (FP64, FastMath)
  const double* grid;          // [GF_COUNT][kall]
  const double* fmtab;         // fast-math tables (nsw6_fastmath.cuh)
  double* const* a;            // not used on device
  // field bases
  double *rhog, *rhogvx, *rhogvy, *rhogvz, *rhogw, *rhoge, *rhogq;
  const double *vx, *vy, *vz;
  double *rho, *tem, *pre, *q, *qd;
  double *precip, *iso1, *iso2;          // [2][lall][gall]: row 1 starts prec_ld doubles after row 0
  size_t prec_ld;                        // lall * gall, or the caller's stride (nsw6_set_precip_stride)
  double *precip_rhoe, *precip_lh_heat, *precip_rhophi, *precip_rhokin;   // [lall][gall]
  double *re_liquid, *re_solid, *re_cld;
  double *rctop, *rwtop, *tctop;         // [lall][1][gall]
  const double* unccn;         // read by the aerosol-indirect switch only
  const double *gsgam2, *gsgam2h, *gam2, *gam2h;
  const double *ix, *iy, *iz, *jx, *jy, *jz;
  const double* z;
  double *GDCLW, *GDCFRC, *GPREC;
  // workspace
  // Sedimenting tracers: ntr = 3 (QR, QS, QG) or 4 with QI sedimentation
  // (QR, QI, QS, QG), in the reference's tracer order.
  int ntr;
  double* zdis;                // [lall][2 ntr][kall][gall]: zdis0 per tracer, then zdis0h per tracer
  unsigned long long* zmax;    // [lall][2 ntr][kall] ordered keys, reset to 0
  unsigned long long* zmin;    // [lall][2 ntr][kall] ordered keys, reset to ~0
  unsigned* satq;              // [1 + lall kall gall]: count (reset to 0), then the saturated cells'
                               // indices l kall gall + k gall + g, for nsw6_satadj_kernel
  DevStatus* status;
};

// The 50 mp_driver array arguments of one call, in the reference order.
struct ArgPtrs {
  double* a[A_COUNT];
};

// Per-thread tapes of the adjoint kernel, interleaved over nslot threads:
// operands pa/pb, partial derivatives da/db and adjoints of cap entries each.
struct TapeMem {
  int* pa;
  int* pb;
  double* da;
  double* db;
  double* adj;
  int nslot, cap, count_only;
};

// Comparisons of doubles on the integer pipe (the FP64 pipe is the scarce one
// on GB300): for non-NaN a and b, a >= b exactly when cmp_key(a) >=
// cmp_key(b), with -0 and +0 equal.
__device__ __forceinline__ long long cmp_key(double x) {
  long long b = __double_as_longlong(x);
  if (b == (long long)0x8000000000000000ULL) b = 0;
  return b < 0 ? (b ^ 0x7fffffffffffffffLL) : b;
}
__device__ __forceinline__ bool is_nan_bits(double x) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
constexpr long long EPS_BITS = 0x3caffffff4178da3LL;   // bit pattern of EPS = 2.220446E-16

__host__ __device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }  // Kokkos::min
__host__ __device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }  // Kokkos::max

// Order-preserving map double -> uint64 (total order, -0 < +0), used for exact
// atomic max/min of the per-level departure-distance extrema.
__host__ __device__ __forceinline__ unsigned long long order_key(double v) {
  union { double d; unsigned long long u; } c;
  c.d = v;
  return (c.u >> 63) ? ~c.u : (c.u | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double key_value(unsigned long long k) {
  union { double d; unsigned long long u; } c;
  c.u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return c.d;
}

}  // namespace nsw6
