// Host driver and C ABI of the GB300 NSW6 step (see include/nsw6.h).
//
// Replaces MP_DRIVER::mp_init / mp_driver (src/mod_mp_driver.cpp:11-24,
// 335-613) and the set-up routines the reference runs through globals:
// GRD_Setup (mod_debug.cpp:92-187), SATURATION_Setup (mod_satadjust.cpp:24-47)
// and mp_nsw6_init (mod_mp_nsw6.cpp:276-434).  All device memory a step needs
// is allocated in nsw6_create; a step enqueues three memsets and three kernels.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>

#include <cuda_runtime.h>

#include "../../include/nsw6.h"
#include "nsw6_common.cuh"
#include "nsw6_fastmath.cuh"

namespace nsw6 {
cudaError_t launch_step(const Problem& P, const Consts& C, cudaStream_t stream, cudaEvent_t* ev,
                        cudaEvent_t before_column = nullptr);
cudaError_t launch_cell_only(const Problem& P, const Consts& C, cudaStream_t stream);
cudaError_t launch_prepare();
cudaError_t launch_serial(const Problem& P, const Consts& C, const ArgPtrs& x, cudaStream_t stream);
cudaError_t launch_tlm(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& dx, const double* params,
                       const double* dparams, cudaStream_t stream);
cudaError_t launch_adj_cellfwd(const Problem& P, const Consts& C, const ArgPtrs& x, double* Y, cudaStream_t stream);
cudaError_t launch_adj_cell(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& xb, const double* YB,
                            const TapeMem& tm, const double* params, double* pbar, int* tape_max, int* done,
                            cudaStream_t stream);
cudaError_t launch_adj_column_staged(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& xb,
                                     const double* Y, double* YB, int ny, double* work, int* bnd, const TapeMem& tm,
                                     int recorded, int mixed, cudaStream_t stream);
cudaError_t launch_adj_cell_hw(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& xb, const double* YB,
                               double* pbar, double* ck, int mixed, cudaStream_t stream);
cudaError_t launch_adj_cell_save(const Problem& P, const Consts& C, const ArgPtrs& x, double* Y, double* ck, int check,
                                 int mixed, cudaStream_t stream);
size_t adj_cell_ck_doubles(int lall, int kall, int gall);
cudaError_t launch_tlm_staged(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& dx,
                              const double* params, const double* dparams, double* Y, double* work, int* bnd,
                              cudaStream_t stream);
int adj_y_fields();
size_t adj_stage_work_doubles(int lall, int kall, int gall);
size_t adj_stage_bound_ints(int lall, int kall);
int adj_stage_tape_cap();
int adj_stage_slots();
int adj_nfields();
constexpr int DERIV_MAX_KALL = 48;   // KA of nsw6_column_step.cuh
constexpr int DERIV_THREADS = 128;   // AD_THREADS of nsw6_ad.cuh
constexpr int ADJ_CELL_SLOTS = 152 * 3 * 128;  // threads of the cell adjoint (3 resident blocks per SM)
cudaError_t launch_math(int fn, const double* x, const double* y, double* out, int n, const double* fmtab,
                        cudaStream_t stream);
}

using namespace nsw6;

struct nsw6_handle {
  int gall = 0, kall = 0, lall_max = 0;
  nsw6_params params{};
  nsw6_options opts{1, 1, 1, 0, 0, 0};
  int opt_active = 0;   // a switch differs from the reference configuration
  Consts C{};
  double* d_grid = nullptr;
  double* d_fmtab = nullptr;
  double* d_zdis = nullptr;
  unsigned long long* d_zmax = nullptr;
  unsigned long long* d_zmin = nullptr;
  unsigned* d_satq = nullptr;   // count and list of the saturated cells of a step
  DevStatus* d_status = nullptr;
  cudaStream_t stream = nullptr;
  int sync_check = 1;
  int itelim = 100;
  int math_lib = 0;   // 0: table-driven exp/log/pow, 1: CUDA libm
  int mixed = 0;      // 0: plain FP64 step, 1: mixed precision, 2: serial-column FP64 (derivative forward)
  // row stride (doubles) of precip / ISO1_precip / ISO2_precip in the per-region
  // calls mp_driver and mp_driver_mixed (0: contiguous [2][gall]); region_call
  // marks such a call while it runs
  long long prec_ld = 0;
  int region_call = 0;
  // derivative kernels: parameters, their adjoint, the tape-size counter and the tapes
  double* d_dparam = nullptr;    // [16]: params [0,7), tangents [8,15)
  double* d_pbar = nullptr;      // [8]
  int* d_tmax = nullptr;
  TapeMem ctape{};       // cell-adjoint tapes
  size_t ctape_bytes = 0;
  TapeMem stape{};       // tapes of the staged column adjoint
  size_t stape_bytes = 0;
  double* d_swork = nullptr;   // work fields, their adjoints and the seeds of the staged column adjoint
  int* d_sbnd = nullptr;       // flux bounds of the staged column adjoint
  int* d_done = nullptr;       // per-cell flags of the cell adjoint
  double* d_cellck = nullptr;  // checkpoint of the cell physics' costly forward values
  int adj_mode = 0;            // cell-phase adjoint: 0 hand-written, 1 recorded tape
  double* d_Y = nullptr;   // cell-phase outputs and their adjoints [2][nfields][lall_max][kall][gall]
  // captured step graph of mp_driver_steps and what it was captured for
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  double* graph_args[A_COUNT] = {};
  int graph_lall = 0, graph_mixed = -1, graph_math = -1, graph_itelim = 0;
  double graph_dt = 0.0;
  nsw6_params graph_params{};
  nsw6_options graph_opts{};
  // device staging of the 50 arguments for host-memory calls (allocated by the
  // first such call)
  double* d_stage = nullptr;
  size_t stage_count = 0;
  // copy streams and per-chunk events of the pipelined host-memory path
  cudaStream_t s_in = nullptr, s_out = nullptr;
  // captured host-memory pipeline (all arguments in pinned memory) and what it
  // was captured for
  cudaGraphExec_t hgraph = nullptr;
  double* hgraph_args[A_COUNT] = {};
  int hgraph_lall = 0, hgraph_mixed = -1, hgraph_math = -1, hgraph_itelim = 0;
  double hgraph_dt = 0.0;
  nsw6_params hgraph_params{};
  nsw6_options hgraph_opts{};
  cudaEvent_t* ev_in = nullptr;    // a chunk's cell-kernel inputs have arrived
  cudaEvent_t* ev_in2 = nullptr;   // its remaining inputs have arrived
  cudaEvent_t* ev_done = nullptr;
  cudaEvent_t ev_join_in = nullptr, ev_join_out = nullptr;   // the copy streams' ends
  cudaEvent_t ev_start = nullptr;
  // kernel timing: a ring of event triples folded into the sums when full
  int timing = 0;
  static constexpr int kRing = 64;
  cudaEvent_t ev[kRing][3] = {};
  int ev_used = 0;
  double t_sum[2] = {0.0, 0.0};
  int t_steps = 0;
};

extern "C" void nsw6_default_options(nsw6_options* o);

namespace {

// MISC_gammafunc, mod_debug.cpp:332-361.
double gammafunc(double xx) {
  static const double coef[6] = {+76.18009172947146, -86.50532032941677, +24.01409824083091,
                                 -1.231739572450155, +0.1208650973866179E-2, -0.5395239384953E-5};
  double x = xx, y = x, tmp = x + 5.5;
  tmp = tmp - (x + 0.5) * std::log(tmp);
  double ser = 1.000000000190015;
  for (int j = 0; j < 6; ++j) {
    y += 1;
    ser += coef[j] / y;
  }
  return std::exp(-tmp + std::log(2.5066282746310005 * ser / x));
}

// mp_nsw6_init (mod_mp_nsw6.cpp:276-434) with its hard-wired choices (Roh and
// Satoh 2014 snow, explicit ice generation, KK2000 autoconversion,
// beta_gaut = 0), GlobalParams defaults (mod_mp_nsw6.h:16-123), the
// effective-radius constants of mp_nsw6_new::init (:506-517) and
// SATURATION_Setup with EIN_TYPE = "SIMPLE" (mod_satadjust.cpp:24-47).
Consts make_consts(const nsw6_params& p, const nsw6_options& o) {
  Consts c;
  std::memset(&c, 0, sizeof(c));
  const double rho_s = 100.0, rho_g = 400.0;
  // Roh_flag (mod_mp_nsw6.cpp:345-357) changes N0g, As, Bs, Esi, Egi, Egs from
  // their GlobalParams values (mod_mp_nsw6.h:16-123)
  const bool roh = o.roh2014 != 0;
  const double Br = 3.0, Bs = roh ? 2.0 : 3.0, Bg = 3.0, Dr = 0.50, Ds = 0.25, Dg = 0.50;
  c.N0r = 8.E+6;
  c.N0s = 3.E+6;
  c.N0g = roh ? 4.0E+8 : 4.E+6;
  c.Ar = PI * DWATR / 6.0;
  c.As = roh ? 0.069 : PI * rho_s / 6.0;
  c.Ag = PI * rho_g / 6.0;
  c.Esi = roh ? 0.25 : 1.0;
  c.Egi = roh ? 0.0 : 0.1;
  c.Egs = roh ? 0.0 : 1.0;
  c.gamma_sacr = 6.0E-2;
  c.gamma_gacs = 90.E-3;
  c.mi = 4.19E-13;
  c.beta_saut = p.beta_saut;
  c.gamma_saut = 6.0E-2;
  c.qicrt_saut = p.qicrt_saut;
  c.A_frz = 0.66;
  c.B_frz = 100.0;
  c.mi40 = 2.46E-10;
  c.mi50 = 4.80E-10;
  c.Ri50 = 5.E-5;
  c.Nc_ihtr = 300.0;
  c.Di_max = 500.E-6;
  c.Di_a = 11.9;
  c.Cr = p.Cr;
  c.Cs = p.Cs;
  c.Cg = p.Cg;
  c.GAM_1br = gammafunc(1.0 + Br);
  c.GAM_2br = gammafunc(2.0 + Br);
  c.GAM_3br = gammafunc(3.0 + Br);
  c.GAM_3dr = gammafunc(3.0 + Dr);
  c.GAM_6dr = gammafunc(6.0 + Dr);
  c.GAM_1brdr = gammafunc(1.0 + Br + Dr);
  c.GAM_5dr_h = gammafunc(0.5 * (5.0 + Dr));
  c.GAM_1bs = gammafunc(1.0 + Bs);
  c.GAM_2bs = gammafunc(2.0 + Bs);
  c.GAM_3bs = gammafunc(3.0 + Bs);
  c.GAM_3ds = gammafunc(3.0 + Ds);
  c.GAM_1bsds = gammafunc(1.0 + Bs + Ds);
  c.GAM_5ds_h = gammafunc(0.5 * (5.0 + Ds));
  c.GAM_1bg = gammafunc(1.0 + Bg);
  c.GAM_3dg = gammafunc(3.0 + Dg);
  c.GAM_1bgdg = gammafunc(1.0 + Bg + Dg);
  c.GAM_5dg_h = gammafunc(0.5 * (5.0 + Dg));
  c.ln10 = std::log(10.0);
  static const double ca[10] = {5.065339, -0.062659, -3.032362, 0.029469, -0.000285,
                                0.31255, 0.000204, 0.003199, 0.0, -0.015952};
  static const double cb[10] = {0.476221, -0.015896, 0.165977, 0.007468, -0.000141,
                                0.060366, 0.000079, 0.000594, 0.0, -0.003577};
  std::memcpy(c.coef_a, ca, sizeof(ca));
  std::memcpy(c.coef_b, cb, sizeof(cb));
  c.Nc_def = 50.0;
  {
    const double Dc = 0.146 - 5.964E-2 * std::log(c.Nc_def / 2000.0);
    const double dgamma_a = 0.1444 / (Dc * Dc);
    const double GAM_dgam = gammafunc(dgamma_a);
    const double GAM_dgam23 = gammafunc(dgamma_a + 2.0 / 3.0);
    c.coef_dgam = GAM_dgam23 / GAM_dgam * std::pow(dgamma_a, (-2.0 / 3.0));
    c.coef_xf = 3.0 / 4.0 / PI / DWATR;
    c.Dc_berry = Dc;
  }
  c.ice_nuc = p.ice_nuc;
  c.kk_aut = p.kk_aut;
  c.LovR_liq = LHV0 / RVAP;
  c.LovR_ice = LHS0 / RVAP;
  c.RTEM00 = 1.0 / TEM00;
  c.dtemp_criteria = std::pow(10.0, (double)(-(15 + 1) / 2));
  c.log_mi50 = std::log(c.mi50);
  c.log_mi40 = std::log(c.mi40);
  c.pow_Nc_m179 = std::pow(c.Nc_def, -1.79);
  c.ln1000 = std::log(1000.0);
  // mod_mp_nsw6.cpp:1205-1208 at rhoqi = max(dens * qi, EPS) = EPS: the number
  // 5.38e7 EPS^0.75 is far below the floor 1e3, so XNi = 1e3 exactly
  c.XNi_eps = std::min(std::max(5.38E+7 * std::pow(EPS, 0.75), 1.0E+3), 1.0E+6);
  c.Di_eps = std::min(c.Di_a * std::sqrt(EPS / c.XNi_eps), c.Di_max);

  // folded constant factors (nsw6_cell.cuh); GAM = GAM_2 = 1, GAM_3 = 2,
  // Esw = Egw = Eri = Esr = Egr = 1 (mod_mp_nsw6.h:58-67, mp_nsw6_init :345-356)
  const double GAM = 1.0, GAM_2 = 1.0, GAM_3 = 2.0;
  c.K_rlmdr = 1.0 / (c.Ar * c.N0r * c.GAM_1br);
  c.K_rlmdg = 1.0 / (c.Ag * c.N0g * c.GAM_1bg);
  c.rAs = 1.0 / c.As;
  c.K_vtr = -c.Cr * c.GAM_1brdr / c.GAM_1br;
  c.K_vts = -c.Cs;
  c.K_vtg = -c.Cg * c.GAM_1bgdg / c.GAM_1bg;
  c.K_sacw = 0.25 * PI * c.Cs;
  c.K_gacw = 0.25 * PI * c.N0g * c.Cg * c.GAM_3dg;
  c.K_raci = 0.25 * PI * c.N0r * c.Cr * c.GAM_3dr;
  c.K_saci = 0.25 * PI * c.Cs;
  c.K_iacr = c.Ar / c.mi * 0.25 * PI * c.N0r * c.Cr * c.GAM_6dr;
  c.K_sacr = c.Ar * 0.25 * PI * c.N0r;
  c.K_2gam2br = 2.0 * c.GAM_2br;
  c.K_gacr = c.Ar * 0.25 * PI * c.N0g * c.N0r;
  c.K_g13 = c.GAM_1br * GAM_3;
  c.K_g22 = 2.0 * c.GAM_2br * GAM_2;
  c.K_racs = c.As * 0.25 * PI * c.N0r;
  c.K_aut = c.kk_aut * c.pow_Nc_m179;
  c.rLHF0 = 1.0 / LHF0;
  c.K_ventr1 = 0.78 * GAM_2;
  c.K_ventr2 = 0.27 * c.GAM_5dr_h;
  c.K_revp = 2.0 * PI * c.N0r;
  c.K_ihtr = c.B_frz / (DWATR * (c.Nc_ihtr * 1.0E+6));
  c.K_vents2 = 0.39 * std::sqrt(c.Cs);
  c.K_2pi = 2.0 * PI;
  c.K_clf = CL / LHF0;
  c.K_ventg1 = 0.78 * GAM_2;
  c.K_ventg2 = 0.27 * c.GAM_5dg_h;
  c.K_gdep = 2.0 * PI * c.N0g;
  c.K_gfrz = 2.0 * PI * c.N0r * 60.0 * c.B_frz * c.Ar;
  c.K_xf = 1.0E-9 / c.Nc_def;
  c.K_r2c = c.coef_dgam * (c.Nc_def * 1.0E+6);
  c.K_r2r = 0.25 * c.N0r * GAM_3;
  // Roh and Satoh (2014) moments (mod_mp_nsw6.cpp:994-1057): loga(nm, t) and
  // b(nm, t) expanded as cubics in t = tems for nm = 0, 1, 2, 3, 4, 2.25, 1.625
  static const double nms[7] = {0.0, 1.0, 2.0, 3.0, 4.0, 2.25, 1.625};
  for (int i = 0; i < 7; ++i) {
    const double nm = nms[i];
    const double* A = c.coef_a;
    const double* B = c.coef_b;
    const double ea[4] = {A[0] + nm * (A[2] + nm * (A[5] + nm * A[9])), A[1] + nm * (A[3] + nm * A[7]),
                          A[4] + nm * A[6], A[8]};
    const double eb[4] = {B[0] + nm * (B[2] + nm * (B[5] + nm * B[9])), B[1] + nm * (B[3] + nm * B[7]),
                          B[4] + nm * B[6], B[8]};
    for (int j = 0; j < 4; ++j) {
      c.roh_a[4 * i + j] = c.ln10 * ea[j];
      c.roh_b[4 * i + j] = eb[j];
    }
  }
  // the switches and the constants of the switched branches (nsw6_cell.cuh)
  c.opt_roh = roh ? 1.0 : 0.0;
  c.opt_expice = (roh || o.explicit_icegen) ? 1.0 : 0.0;   // mp_nsw6_init forces it with Roh_flag
  c.opt_kk = o.kk2000 ? 1.0 : 0.0;
  c.opt_qised = o.qi_sediment ? 1.0 : 0.0;
  c.opt_kin2kin = o.kin2kin ? 1.0 : 0.0;
  c.opt_indir = o.aerosol_indirect ? 1.0 : 0.0;
  c.K_gaci = 0.25 * PI * c.Egi * c.N0g * c.Cg * c.GAM_3dg;
  c.K_gacs = c.As * 0.25 * PI * c.N0g;
  c.K_rlmds = 1.0 / (c.As * c.N0s * c.GAM_1bs);
  c.K_m0 = c.N0s * GAM;
  c.K_m1 = c.N0s * GAM_2;
  c.K_m2 = c.N0s * GAM_3;
  c.K_m0bs = c.N0s * c.GAM_1bs;
  c.K_m1bs = c.N0s * c.GAM_2bs;
  c.K_m2bs = c.N0s * c.GAM_3bs;
  c.K_m2ds = c.N0s * c.GAM_3ds;
  c.K_m5dsh = c.N0s * c.GAM_5ds_h;
  c.K_rmomvt = c.GAM_1bsds / c.GAM_1bs;
  // Bergeron_param tables (mod_mp_nsw6.cpp:1845-1861)
  static const double a1t[32] = {0.0001E-7, 0.7939E-7, 0.7841E-6, 0.3369E-5, 0.4336E-5, 0.5285E-5, 0.3728E-5,
                                 0.1852E-5, 0.2991E-6, 0.4248E-6, 0.7434E-6, 0.1812E-5, 0.4394E-5, 0.9145E-5,
                                 0.1725E-4, 0.3348E-4, 0.1725E-4, 0.9175E-5, 0.4412E-5, 0.2252E-5, 0.9115E-6,
                                 0.4876E-6, 0.3473E-6, 0.4758E-6, 0.6306E-6, 0.8573E-6, 0.7868E-6, 0.7192E-6,
                                 0.6513E-6, 0.5956E-6, 0.5333E-6, 0.4834E-6};
  static const double a2t[32] = {0.0100, 0.4006, 0.4831, 0.5320, 0.5307, 0.5319, 0.5249, 0.4888,
                                 0.3849, 0.4047, 0.4318, 0.4771, 0.5183, 0.5463, 0.5651, 0.5813,
                                 0.5655, 0.5478, 0.5203, 0.4906, 0.4447, 0.4126, 0.3960, 0.4149,
                                 0.4320, 0.4506, 0.4483, 0.4460, 0.4433, 0.4413, 0.4382, 0.4361};
  std::memcpy(c.berg_a1, a1t, sizeof(a1t));
  std::memcpy(c.berg_a2, a2t, sizeof(a2t));
  const double Eiw = 1.0, vti50 = 1.0;
  c.K_berg_w = PI * Eiw * c.Ri50 * c.Ri50 * vti50;
  c.sat_ulimit = 273.16;   // SATURATION_Setrange of the ice_adjust branch, :657-658
  c.sat_llimit = 233.16;
  return c;
}

Consts make_consts(const nsw6_params& p) {
  nsw6_options o;
  nsw6_default_options(&o);
  return make_consts(p, o);
}

// Fast-math tables (nsw6_fastmath.cuh), computed in extended precision:
// [0,256) 2^(j/256) rounded; [256,512) its relative rounding error;
// [512,768) 1/c_j; [768,1024) -log(1/c_j), where c_j is the centre of the j-th
// of 256 mantissa intervals of [0.75, 1.5).
void build_fastmath_tables(double* t) {
  for (int j = 0; j < FM_EXP_N; ++j) {
    const long double v = exp2l((long double)j / 256.0L);
    t[j] = (double)v;
    t[FM_EXP_N + j] = (double)(v / (long double)t[j] - 1.0L);
  }
  double* ic_t = t + 2 * FM_EXP_N;
  double* lc_t = ic_t + FM_LOG_N;
  for (int j = 0; j < FM_LOG_N; ++j) {
    unsigned long long lo_bits = 0x3FE8000000000000ull + ((unsigned long long)j << 44);
    unsigned long long hi_bits = lo_bits + (1ull << 44);
    double mlo, mhi;
    std::memcpy(&mlo, &lo_bits, 8);
    std::memcpy(&mhi, &hi_bits, 8);
    const long double cj = 0.5L * ((long double)mlo + (long double)mhi);
    const double ic = (double)(1.0L / cj);
    ic_t[j] = ic;
    lc_t[j] = (double)(-logl((long double)ic));
  }
}

// GRD_Setup, mod_debug.cpp:92-187, plus GRD_gz_shift (mod_precip_transport.cpp:698-709).
void make_grid(int K, const double* gz, const double* gzh, double* out /* [GF_COUNT][K] */) {
  std::memset(out, 0, sizeof(double) * GF_COUNT * (size_t)K);
  double* g_gz = out + GF_GZ * K;
  double* g_gzh = out + GF_GZH * K;
  double* dgz = out + GF_DGZ * K;
  double* dgzh = out + GF_DGZH * K;
  double* rdgz = out + GF_RDGZ * K;
  double* rdgzh = out + GF_RDGZH * K;
  double* af = out + GF_AFACT * K;
  double* bf = out + GF_BFACT * K;
  double* cf = out + GF_CFACT * K;
  double* df = out + GF_DFACT * K;
  double* gzs = out + GF_GZSHIFT * K;
  const int kmin = 1, kmax = K - 2;
  for (int k = 0; k < K; ++k) {
    g_gz[k] = gz[k];
    g_gzh[k] = gzh[k];
  }
  for (int k = kmin - 1; k <= kmax; ++k) dgz[k] = g_gzh[k + 1] - g_gzh[k];
  dgz[kmax + 1] = dgz[kmax];
  for (int k = kmin; k <= kmax + 1; ++k) dgzh[k] = g_gz[k] - g_gz[k - 1];
  dgzh[kmin - 1] = dgzh[kmin];
  for (int k = 0; k < K; ++k) {
    rdgz[k] = 1.0 / dgz[k];
    rdgzh[k] = 1.0 / dgzh[k];
  }
  for (int k = kmin; k <= kmax + 1; ++k) af[k] = (g_gzh[k] - g_gz[k - 1]) / (g_gz[k] - g_gz[k - 1]);
  af[kmin - 1] = 1.0;
  for (int k = 0; k < K; ++k) bf[k] = 1.0 - af[k];
  for (int k = kmin; k <= kmax; ++k) cf[k] = (g_gz[k] - g_gzh[k]) / (g_gzh[k + 1] - g_gzh[k]);
  cf[kmin - 1] = 1.0;
  cf[kmax + 1] = 0.0;
  for (int k = 0; k < K; ++k) df[k] = 1.0 - cf[k];
  for (int k = kmin; k <= kmax + 1; ++k) gzs[k] = g_gz[k - 1];
  double* rdzs = out + GF_RDZS * K;
  double* rdzsh = out + GF_RDZSH * K;
  for (int k = 1; k < K; ++k) {
    rdzs[k] = 1.0 / (dgz[k - 1] + dgz[k]);
    rdzsh[k] = 1.0 / (dgzh[k - 1] + dgzh[k]);
  }
}

// Elements per region of each mp_driver argument (reference order).
size_t arg_region_elems(int a, int K, int G) {
  switch (a) {
    case A_rhogq:
    case A_q:
      return (size_t)NQ * K * G;
    case A_precip:
    case A_ISO1:
    case A_ISO2:
      return 2 * (size_t)G;
    case A_precip_rhoe:
    case A_precip_lh_heat:
    case A_precip_rhophi:
    case A_precip_rhokin:
    case A_rctop:
    case A_rwtop:
    case A_tctop:
    case A_ix:
    case A_iy:
    case A_iz:
    case A_jx:
    case A_jy:
    case A_jz:
      return (size_t)G;
    default:
      return (size_t)K * G;
  }
}

// Arguments the step reads (copied to the device by host-memory calls) and
// writes (copied back).
bool arg_is_read(int a) {
  switch (a) {
    case A_rhog: case A_rhogvx: case A_rhogvy: case A_rhogvz: case A_rhogw: case A_rhoge: case A_rhogq:
    case A_vx: case A_vy: case A_vz: case A_tem: case A_q: case A_gsgam2: case A_gsgam2h: case A_gam2:
    case A_gam2h: case A_ix: case A_iy: case A_iz: case A_jx: case A_jy: case A_jz: case A_z:
      return true;
    default:
      return false;
  }
}
// Arguments the cell kernel reads or writes in place (the host pipeline copies
// them in before the rest).
bool cell_phase_arg(int a) {
  switch (a) {
    case A_rhog: case A_rhoge: case A_tem: case A_rhogq: case A_q: case A_gsgam2: case A_unccn:
      return true;
    default:
      return false;
  }
}
bool arg_is_written(int a) {
  switch (a) {
    case A_rhog: case A_rhogvx: case A_rhogvy: case A_rhogvz: case A_rhogw: case A_rhoge: case A_rhogq:
    case A_rho: case A_tem: case A_pre: case A_q: case A_qd: case A_precip: case A_ISO1: case A_ISO2:
    case A_precip_rhoe: case A_precip_lh_heat: case A_precip_rhophi: case A_precip_rhokin: case A_re_liquid:
    case A_re_solid: case A_re_cld: case A_rctop: case A_rwtop: case A_tctop: case A_GDCLW: case A_GDCFRC:
    case A_GPREC:
      return true;
    default:
      return false;
  }
}

int fill_problem(nsw6_handle* h, int lall, double* const* a, double dt, Problem& P) {
  if (!h || lall < 1 || lall > h->lall_max || !a) return NSW6_ERR_BAD_ARG;
  if (!(dt > 0.0) || !std::isfinite(dt)) return NSW6_ERR_BAD_ARG;
  for (int i = 0; i < A_COUNT; ++i) {
    if (arg_is_read(i) || arg_is_written(i)) {
      if (!a[i]) return NSW6_ERR_BAD_ARG;
    }
  }
  std::memset(&P, 0, sizeof(P));
  P.gall = h->gall;
  P.kall = h->kall;
  P.kmin = 1;
  P.kmax = h->kall - 2;
  P.lall = lall;
  P.prec_ld = (h->region_call && h->prec_ld > 0) ? (size_t)h->prec_ld : (size_t)lall * (size_t)h->gall;
  P.dt = dt;
  P.dt2 = std::pow(dt, 2);
  P.dt3 = std::pow(dt, 3);
  P.hdt2 = P.dt2 / 2.0;
  P.sdt3 = P.dt3 / 6.0;
  P.itelim = h->itelim;
  P.grid = h->d_grid;
  P.fmtab = h->d_fmtab;
  P.rdt = 1.0 / dt;
  P.math_lib = h->math_lib;
  P.mixed = h->mixed;
  P.opt = h->opt_active;
  P.ntr = h->opts.qi_sediment ? 4 : 3;
  // the switches run in the FP64 and mixed-precision kernels (FastMath)
  if (h->opt_active && (h->mixed == 2 || h->math_lib != 0)) return NSW6_ERR_UNSUPPORTED;
  if (h->opts.aerosol_indirect && !a[A_unccn]) return NSW6_ERR_BAD_ARG;
  P.unccn = a[A_unccn];
  P.rhog = a[A_rhog];
  P.rhogvx = a[A_rhogvx];
  P.rhogvy = a[A_rhogvy];
  P.rhogvz = a[A_rhogvz];
  P.rhogw = a[A_rhogw];
  P.rhoge = a[A_rhoge];
  P.rhogq = a[A_rhogq];
  P.vx = a[A_vx];
  P.vy = a[A_vy];
  P.vz = a[A_vz];
  P.rho = a[A_rho];
  P.tem = a[A_tem];
  P.pre = a[A_pre];
  P.q = a[A_q];
  P.qd = a[A_qd];
  P.precip = a[A_precip];
  P.iso1 = a[A_ISO1];
  P.iso2 = a[A_ISO2];
  P.precip_rhoe = a[A_precip_rhoe];
  P.precip_lh_heat = a[A_precip_lh_heat];
  P.precip_rhophi = a[A_precip_rhophi];
  P.precip_rhokin = a[A_precip_rhokin];
  P.re_liquid = a[A_re_liquid];
  P.re_solid = a[A_re_solid];
  P.re_cld = a[A_re_cld];
  P.rctop = a[A_rctop];
  P.rwtop = a[A_rwtop];
  P.tctop = a[A_tctop];
  P.gsgam2 = a[A_gsgam2];
  P.gsgam2h = a[A_gsgam2h];
  P.gam2 = a[A_gam2];
  P.gam2h = a[A_gam2h];
  P.ix = a[A_ix];
  P.iy = a[A_iy];
  P.iz = a[A_iz];
  P.jx = a[A_jx];
  P.jy = a[A_jy];
  P.jz = a[A_jz];
  P.z = a[A_z];
  P.GDCLW = a[A_GDCLW];
  P.GDCFRC = a[A_GDCFRC];
  P.GPREC = a[A_GPREC];
  P.zdis = h->d_zdis;
  P.zmax = h->d_zmax;
  P.zmin = h->d_zmin;
  P.satq = h->d_satq;
  P.status = h->d_status;
  return NSW6_OK;
}

// Adds the elapsed times of the recorded event triples to the sums.
int fold_timing(nsw6_handle* h) {
  if (h->ev_used == 0) return NSW6_OK;
  if (cudaEventSynchronize(h->ev[h->ev_used - 1][2]) != cudaSuccess) return NSW6_ERR_CUDA;
  for (int i = 0; i < h->ev_used; ++i) {
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, h->ev[i][0], h->ev[i][1]);
    cudaEventElapsedTime(&b, h->ev[i][1], h->ev[i][2]);
    h->t_sum[0] += a;
    h->t_sum[1] += b;
  }
  h->t_steps += h->ev_used;
  h->ev_used = 0;
  return NSW6_OK;
}

cudaEvent_t* next_events(nsw6_handle* h) {
  if (!h->timing) return nullptr;
  if (h->ev_used == nsw6_handle::kRing && fold_timing(h) != NSW6_OK) return nullptr;
  cudaEvent_t* e = h->ev[h->ev_used];
  if (!e[0]) {
    for (int j = 0; j < 3; ++j)
      if (cudaEventCreate(&e[j]) != cudaSuccess) return nullptr;
  }
  ++h->ev_used;
  return e;
}

int finish(nsw6_handle* h, cudaError_t launch) {
  if (launch != cudaSuccess) return NSW6_ERR_CUDA;
  if (!h->sync_check) return NSW6_OK;
  return nsw6_last_error(h, nullptr, nullptr, nullptr, nullptr);
}

// Device staging area for all 50 arguments of lall_max regions (the host
// entry copies through it; the derivative kernels' pre-pass runs on it).
int ensure_stage(nsw6_handle* h, double** dev) {
  const int K = h->kall, G = h->gall;
  size_t need = 0;
  for (int i = 0; i < A_COUNT; ++i) need += arg_region_elems(i, K, G) * (size_t)h->lall_max;
  if (!h->d_stage) {
    if (cudaMalloc(&h->d_stage, sizeof(double) * need) != cudaSuccess) return NSW6_ERR_CUDA;
    h->stage_count = need;
  }
  size_t offs = 0;
  for (int i = 0; i < A_COUNT; ++i) {
    dev[i] = h->d_stage + offs;
    offs += arg_region_elems(i, K, G) * (size_t)h->lall_max;
  }
  return NSW6_OK;
}

// Region extrema of the departure distances of state a (into d_zmax/d_zmin):
// the FP64 cell kernel on a copy of the fields it updates.
int deriv_prepass(nsw6_handle* h, int lall, double* const* a, double dt) {
  double* dev[A_COUNT];
  int rc = ensure_stage(h, dev);
  if (rc != NSW6_OK) return rc;
  double* pa[A_COUNT];
  for (int i = 0; i < A_COUNT; ++i) pa[i] = dev[i];
  const int copy[4] = {A_rhog, A_tem, A_q, A_rhogq};
  for (int c = 0; c < 4; ++c) {
    const int i = copy[c];
    if (!a[i]) return NSW6_ERR_BAD_ARG;
    const size_t bytes = sizeof(double) * arg_region_elems(i, h->kall, h->gall) * (size_t)lall;
    if (cudaMemcpyAsync(dev[i], a[i], bytes, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess)
      return NSW6_ERR_CUDA;
  }
  pa[A_gsgam2] = a[A_gsgam2];
  Problem P;
  rc = fill_problem(h, lall, pa, dt, P);
  if (rc != NSW6_OK) return rc;
  return launch_cell_only(P, h->C, h->stream) == cudaSuccess ? NSW6_OK : NSW6_ERR_CUDA;
}

// serial: the call runs the serial column step (one column per thread, at
// most DERIV_MAX_KALL levels, no scheme switch); the staged derivative
// kernels take any kall and every scheme switch (Berry warm rain, the aerosol
// effect, the classic snow moments, the Bergeron process with the mixed-phase
// saturation adjustment, QI sedimentation, KIN2KIN).
int deriv_check(nsw6_handle* h, int lall, double* const* a, double* const* b, bool serial) {
  if (!h || !a || !b || lall < 1 || lall > h->lall_max) return NSW6_ERR_BAD_ARG;
  if ((serial && h->kall > DERIV_MAX_KALL) || (h->opt_active && serial)) return NSW6_ERR_UNSUPPORTED;
  for (int i = 0; i < A_COUNT; ++i)
    if ((arg_is_read(i) || arg_is_written(i)) && (!a[i] || !b[i])) return NSW6_ERR_BAD_ARG;
  if (!h->d_dparam) {
    if (cudaMalloc(&h->d_dparam, sizeof(double) * 16) != cudaSuccess ||
        cudaMalloc(&h->d_pbar, sizeof(double) * 8) != cudaSuccess ||
        cudaMalloc(&h->d_tmax, sizeof(int)) != cudaSuccess)
      return NSW6_ERR_CUDA;
  }
  return NSW6_OK;
}

// Cell-phase outputs and their tangents / adjoints (Y), the staged column
// work fields, flux bounds and per-cell flags, sized for lall_max, kept in the
// handle.
int ensure_adj_work(nsw6_handle* h) {
  if (adj_y_fields() != adj_nfields()) return NSW6_ERR_UNSUPPORTED;   // the two layouts of Y must agree
  const size_t NC = (size_t)h->lall_max * h->kall * h->gall;
  if (!h->d_Y && cudaMalloc(&h->d_Y, sizeof(double) * 2 * adj_nfields() * NC) != cudaSuccess) return NSW6_ERR_CUDA;
  if (!h->d_swork) {
    if (cudaMalloc(&h->d_swork, sizeof(double) * adj_stage_work_doubles(h->lall_max, h->kall, h->gall)) !=
            cudaSuccess ||
        cudaMalloc(&h->d_sbnd, sizeof(int) * adj_stage_bound_ints(h->lall_max, h->kall)) != cudaSuccess ||
        cudaMalloc(&h->d_done, sizeof(int) * NC) != cudaSuccess)
      return NSW6_ERR_CUDA;
  }
  return NSW6_OK;
}

int run_serial(nsw6_handle* h, int lall, double* const* a, double dt) {
  if (h->kall > DERIV_MAX_KALL || h->opt_active) return NSW6_ERR_UNSUPPORTED;
  int rc = deriv_prepass(h, lall, a, dt);
  if (rc != NSW6_OK) return rc;
  Problem P;
  rc = fill_problem(h, lall, a, dt, P);
  if (rc != NSW6_OK) return rc;
  ArgPtrs x;
  for (int i = 0; i < A_COUNT; ++i) x.a[i] = a[i];
  return finish(h, launch_serial(P, h->C, x, h->stream));
}

// Host-memory arrays: the regions are independent, so the call runs in
// chunks of regions over three streams, the copy-in of chunk j+1 and the
// copy-out of chunk j-1 overlapping the step of chunk j (the H2D and D2H copy
// engines and the SMs all busy).  Each chunk's step is the batched step on the
// chunk's regions; the precipitation outputs ([2][lall][gall] in the caller's
// layout) are staged per chunk as [2][chunk][gall] and copied back in two
// pieces.  Returns after all copies are done.
// Enqueues the host-memory step as a pipeline of chunks of regions: copies in
// on s_in, the step on cs, copies out on s_out, from an event recorded on cs;
// cs ends waiting for both copy streams.  rc: a fill_problem error.
// Doubles of argument i the host entry copies in for nl regions: every
// argument the step reads, whole, except two it reads in part.  Of q only QV
// is read (the cell kernel's input; QC..QG of every level are formed from
// rhogq), of rhoge only the two halo levels (the cell kernel forms the
// interior levels' from tem, rhog and q before anything reads them).  The
// device staging keeps whatever the skipped parts held; nothing reads them.
size_t host_in_doubles(const nsw6_handle* h, int i, int nl) {
  const size_t K = h->kall, G = h->gall;
  if (!arg_is_read(i) && !(i == A_unccn && h->opts.aerosol_indirect)) return 0;
  if (i == A_q) return K * G * (size_t)nl;
  if (i == A_rhoge) return 2 * G * (size_t)nl;
  return arg_region_elems(i, (int)K, (int)G) * (size_t)nl;
}

cudaError_t enqueue_host(nsw6_handle* h, int lall, double* const* args, double* const* dev, double dt, cudaStream_t cs,
                         int& rc) {
  const int K = h->kall, G = h->gall;
  rc = NSW6_OK;
  if (cudaEventRecord(h->ev_start, cs) != cudaSuccess || cudaStreamWaitEvent(h->s_in, h->ev_start, 0) != cudaSuccess)
    return cudaErrorUnknown;
  // Chunks of regions: the first chunk's copy in and the last chunk's copy
  // out are not hidden behind compute, so those two are one region each; the
  // FP64 step (compute above the copies) takes the rest in about four chunks
  // (larger launches fill the GPU's last wave better), the mixed-precision
  // step (copies above the compute) one region at a time, so that each
  // region's copy out starts as soon as it is done.
  const int mid = (lall > 2 && h->mixed != 1) ? (lall - 2 + 3) / 4 : 1;
  auto chunk_len = [&](int l0) {
    if (lall <= 2 || l0 == 0 || l0 == lall - 1) return 1;
    const int left = lall - 1 - l0;   // regions before the last one
    return left < mid ? left : mid;
  };
  cudaError_t err = cudaSuccess;
  int nchunk = 0;
  for (int l0 = 0, nl = 0; l0 < lall && err == cudaSuccess; l0 += nl, ++nchunk) {
    nl = chunk_len(l0);
    // chunk views: region l0 of every array (the precipitation outputs at
    // their own [2][nl][gall] block of the staging)
    double* cdev[A_COUNT];
    double* chost[A_COUNT];
    for (int i = 0; i < A_COUNT; ++i) {
      const size_t e = arg_region_elems(i, K, G);
      cdev[i] = dev[i] + e * (size_t)l0;
      chost[i] = args[i] ? args[i] + ((i == A_precip || i == A_ISO1 || i == A_ISO2) ? (size_t)l0 * G : e * l0)
                         : nullptr;
    }
    // inputs in two groups: first what the cell kernel reads or rewrites in
    // place, then what only the column kernel reads, which arrives while the
    // cell kernel runs; of q and rhoge only the parts the step reads
    // (host_in_doubles)
    for (int group = 0; group < 2 && err == cudaSuccess; ++group) {
      for (int i = 0; i < A_COUNT && err == cudaSuccess; ++i) {
        if (host_in_doubles(h, i, 1) == 0) continue;
        if ((cell_phase_arg(i) ? 0 : 1) != group) continue;
        const size_t e = arg_region_elems(i, K, G);
        // nl blocks of n doubles, one per region, e doubles apart: one 2D copy
        // (its pitch is limited to 2^31 - 1 bytes), else one copy per region
        auto copy_blocks = [&](size_t o, size_t n) {
          if (sizeof(double) * e <= (size_t)INT_MAX)
            return cudaMemcpy2DAsync(cdev[i] + o, sizeof(double) * e, chost[i] + o, sizeof(double) * e,
                                     sizeof(double) * n, nl, cudaMemcpyHostToDevice, h->s_in);
          cudaError_t ce = cudaSuccess;
          for (int r = 0; r < nl && ce == cudaSuccess; ++r)
            ce = cudaMemcpyAsync(cdev[i] + o + e * r, chost[i] + o + e * r, sizeof(double) * n,
                                 cudaMemcpyHostToDevice, h->s_in);
          return ce;
        };
        if (i == A_q) {
          err = copy_blocks(0, (size_t)K * G);   // q[QV] of each region
        } else if (i == A_rhoge) {
          err = copy_blocks(0, G);               // levels 0 and K-1 of each region
          if (err == cudaSuccess) err = copy_blocks((size_t)(K - 1) * G, G);
        } else {
          err = cudaMemcpyAsync(cdev[i], chost[i], sizeof(double) * e * nl, cudaMemcpyHostToDevice, h->s_in);
        }
      }
      if (err == cudaSuccess) err = cudaEventRecord(group == 0 ? h->ev_in[nchunk] : h->ev_in2[nchunk], h->s_in);
    }
    if (err != cudaSuccess) break;
    if ((err = cudaStreamWaitEvent(cs, h->ev_in[nchunk], 0)) != cudaSuccess) break;
    Problem P;
    rc = fill_problem(h, nl, cdev, dt, P);
    if (rc != NSW6_OK) break;
    if ((err = launch_step(P, h->C, cs, nullptr, h->ev_in2[nchunk])) != cudaSuccess) break;
    if ((err = cudaEventRecord(h->ev_done[nchunk], cs)) != cudaSuccess) break;
    if ((err = cudaStreamWaitEvent(h->s_out, h->ev_done[nchunk], 0)) != cudaSuccess) break;
    for (int i = 0; i < A_COUNT && err == cudaSuccess; ++i) {
      if (!arg_is_written(i)) continue;
      if (i == A_precip || i == A_ISO1 || i == A_ISO2) {
        // [2][nl][G] staged -> rows 0 and 1 of the caller's [2][lall][G]
        err = cudaMemcpyAsync(chost[i], cdev[i], sizeof(double) * nl * G, cudaMemcpyDeviceToHost, h->s_out);
        if (err == cudaSuccess)
          err = cudaMemcpyAsync(chost[i] + (size_t)lall * G, cdev[i] + (size_t)nl * G, sizeof(double) * nl * G,
                                cudaMemcpyDeviceToHost, h->s_out);
      } else {
        err = cudaMemcpyAsync(chost[i], cdev[i], sizeof(double) * arg_region_elems(i, K, G) * nl,
                              cudaMemcpyDeviceToHost, h->s_out);
      }
    }
  }
  // cs waits for the last copies out (and the copy-in stream, which ended before them)
  if (err == cudaSuccess && rc == NSW6_OK) {
    if ((err = cudaEventRecord(h->ev_join_out, h->s_out)) == cudaSuccess &&
        (err = cudaEventRecord(h->ev_join_in, h->s_in)) == cudaSuccess &&
        (err = cudaStreamWaitEvent(cs, h->ev_join_out, 0)) == cudaSuccess)
      err = cudaStreamWaitEvent(cs, h->ev_join_in, 0);
  }
  return err;
}

// True when every argument the host entry copies is in page-locked memory
// (a stream capture takes copies from page-locked memory only).
bool host_args_pinned(nsw6_handle* h, double* const* args) {
  for (int i = 0; i < A_COUNT; ++i) {
    if (!args[i] || !(arg_is_read(i) || arg_is_written(i) || (i == A_unccn && h->opts.aerosol_indirect))) continue;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, args[i]) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (at.type != cudaMemoryTypeHost) return false;
  }
  return true;
}

int run_host(nsw6_handle* h, int lall, double* const* args, double dt) {
  // precision 2, the serial check path, runs on device arrays only (its
  // pre-pass uses the staging buffers this entry copies into)
  if (h->mixed == 2) return NSW6_ERR_UNSUPPORTED;
  for (int i = 0; i < A_COUNT; ++i)
    if ((arg_is_read(i) || arg_is_written(i)) && !args[i]) return NSW6_ERR_BAD_ARG;
  if (h->opts.aerosol_indirect && !args[A_unccn]) return NSW6_ERR_BAD_ARG;
  if (!(dt > 0.0) || !std::isfinite(dt)) return NSW6_ERR_BAD_ARG;
  double* dev[A_COUNT];
  int rc = ensure_stage(h, dev);
  if (rc != NSW6_OK) return rc;
  if (!h->s_in) {
    if (cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_start, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join_out, cudaEventDisableTiming) != cudaSuccess)
      return NSW6_ERR_CUDA;
    h->ev_in = new cudaEvent_t[h->lall_max]();
    h->ev_in2 = new cudaEvent_t[h->lall_max]();
    h->ev_done = new cudaEvent_t[h->lall_max]();
    for (int i = 0; i < h->lall_max; ++i)
      if (cudaEventCreateWithFlags(&h->ev_in[i], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&h->ev_in2[i], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&h->ev_done[i], cudaEventDisableTiming) != cudaSuccess)
        return NSW6_ERR_CUDA;
  }
  if (launch_prepare() != cudaSuccess) return NSW6_ERR_CUDA;
  // With the arguments in page-locked memory the pipeline (some 400 copies and
  // launches) is captured once into a CUDA graph and replayed: one launch a
  // step, so that a host thread descheduled while it issues the work does
  // not leave the copy engines and the SMs waiting.  It is re-captured when
  // the arrays, lall, dt, the parameters, the switches or the precision change.
  if (host_args_pinned(h, args)) {
    bool same = h->hgraph && h->hgraph_lall == lall && h->hgraph_dt == dt && h->hgraph_mixed == h->mixed &&
                h->hgraph_math == h->math_lib && h->hgraph_itelim == h->itelim &&
                std::memcmp(&h->hgraph_params, &h->params, sizeof(nsw6_params)) == 0 &&
                std::memcmp(&h->hgraph_opts, &h->opts, sizeof(nsw6_options)) == 0;
    for (int i = 0; same && i < A_COUNT; ++i) same = h->hgraph_args[i] == args[i];
    if (!same) {
      if (h->hgraph) {
        cudaGraphExecDestroy(h->hgraph);
        h->hgraph = nullptr;
      }
      if (!h->cap_stream && cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
        return NSW6_ERR_CUDA;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return NSW6_ERR_CUDA;
      const cudaError_t qe = enqueue_host(h, lall, args, dev, dt, h->cap_stream, rc);
      const cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &g);
      if (rc != NSW6_OK || qe != cudaSuccess || ce != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc != NSW6_OK ? rc : NSW6_ERR_CUDA;
      }
      const cudaError_t ie = cudaGraphInstantiate(&h->hgraph, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) {
        h->hgraph = nullptr;
        return NSW6_ERR_CUDA;
      }
      for (int i = 0; i < A_COUNT; ++i) h->hgraph_args[i] = args[i];
      h->hgraph_lall = lall;
      h->hgraph_dt = dt;
      h->hgraph_mixed = h->mixed;
      h->hgraph_math = h->math_lib;
      h->hgraph_itelim = h->itelim;
      h->hgraph_params = h->params;
      h->hgraph_opts = h->opts;
    }
    if (cudaGraphLaunch(h->hgraph, h->stream) != cudaSuccess) return NSW6_ERR_CUDA;
    return nsw6_last_error(h, nullptr, nullptr, nullptr, nullptr);
  }
  const cudaError_t err = enqueue_host(h, lall, args, dev, dt, h->stream, rc);
  const cudaError_t se = cudaStreamSynchronize(h->stream);
  if (rc != NSW6_OK) return rc;
  if (err != cudaSuccess || se != cudaSuccess) return NSW6_ERR_CUDA;
  return nsw6_last_error(h, nullptr, nullptr, nullptr, nullptr);
}

int run(nsw6_handle* h, int lall, double* const* a, double dt) {
  if (h->mixed == 2) return run_serial(h, lall, a, dt);
  Problem P;
  int rc = fill_problem(h, lall, a, dt, P);
  if (rc != NSW6_OK) return rc;
  return finish(h, launch_step(P, h->C, h->stream, next_events(h)));
}

}  // namespace

extern "C" {

void nsw6_default_params(nsw6_params* p) {
  if (!p) return;
  p->beta_saut = 5.0E-3;
  p->qicrt_saut = 0.0;
  p->Cr = 130.0;
  p->Cs = 4.84;
  p->Cg = std::sqrt((4.0 * 400.0 * GRAV) / (3.0 * DENS00 * 0.6));
  p->ice_nuc = 4.92E-11;
  p->kk_aut = 1350.0;
}

int nsw6_create(nsw6_handle** out, int gall, int kall, int lall_max, const double* gz, const double* gzh) {
  if (!out || gall < 1 || kall < 5 || kall > MAX_KALL || lall_max < 1 || !gz || !gzh) return NSW6_ERR_BAD_ARG;
  // the saturated cells of a step are listed by 32-bit cell index
  if ((unsigned long long)gall * kall * lall_max >= 0xFFFFFFFFull) return NSW6_ERR_TOO_LARGE;
  *out = nullptr;
  nsw6_handle* h = new (std::nothrow) nsw6_handle();
  if (!h) return NSW6_ERR_BAD_ARG;
  h->gall = gall;
  h->kall = kall;
  h->lall_max = lall_max;
  nsw6_default_params(&h->params);
  h->C = make_consts(h->params);
  double* hgrid = (double*)std::malloc(sizeof(double) * (GF_COUNT * (size_t)kall + FM_TABLE_DOUBLES));
  make_grid(kall, gz, gzh, hgrid);
  double* htab = hgrid + GF_COUNT * (size_t)kall;
  build_fastmath_tables(htab);
  const size_t KG = (size_t)kall * gall;
  // departure distances and extrema: 2 rows per sedimenting tracer, up to 4
  // tracers with QI sedimentation
  const size_t nkey = (size_t)lall_max * 8 * kall;
  bool ok = cudaMalloc(&h->d_grid, sizeof(double) * GF_COUNT * kall) == cudaSuccess &&
            cudaMalloc(&h->d_zdis, sizeof(double) * 8 * KG * lall_max) == cudaSuccess &&
            cudaMalloc(&h->d_zmax, sizeof(unsigned long long) * nkey) == cudaSuccess &&
            cudaMalloc(&h->d_zmin, sizeof(unsigned long long) * nkey) == cudaSuccess &&
            cudaMalloc(&h->d_satq, sizeof(unsigned) * (1 + KG * lall_max)) == cudaSuccess &&
            cudaMalloc(&h->d_status, sizeof(DevStatus)) == cudaSuccess &&
            cudaMalloc(&h->d_fmtab, sizeof(double) * FM_TABLE_DOUBLES) == cudaSuccess &&
            cudaMemcpy(h->d_fmtab, htab, sizeof(double) * FM_TABLE_DOUBLES, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(h->d_grid, hgrid, sizeof(double) * GF_COUNT * kall, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemset(h->d_status, 0, sizeof(DevStatus)) == cudaSuccess;
  std::free(hgrid);
  if (!ok) {
    nsw6_destroy(h);
    return NSW6_ERR_CUDA;
  }
  *out = h;
  return NSW6_OK;
}

int nsw6_destroy(nsw6_handle* h) {
  if (!h) return NSW6_OK;
  cudaFree(h->d_grid);
  cudaFree(h->d_fmtab);
  cudaFree(h->d_zdis);
  cudaFree(h->d_zmax);
  cudaFree(h->d_zmin);
  cudaFree(h->d_satq);
  cudaFree(h->d_status);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->hgraph) cudaGraphExecDestroy(h->hgraph);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  if (h->s_in) cudaStreamDestroy(h->s_in);
  if (h->s_out) cudaStreamDestroy(h->s_out);
  for (int i = 0; h->ev_in && i < h->lall_max; ++i) {
    if (h->ev_in[i]) cudaEventDestroy(h->ev_in[i]);
    if (h->ev_in2[i]) cudaEventDestroy(h->ev_in2[i]);
    if (h->ev_done[i]) cudaEventDestroy(h->ev_done[i]);
  }
  delete[] h->ev_in;
  delete[] h->ev_in2;
  delete[] h->ev_done;
  if (h->ev_start) cudaEventDestroy(h->ev_start);
  if (h->ev_join_in) cudaEventDestroy(h->ev_join_in);
  if (h->ev_join_out) cudaEventDestroy(h->ev_join_out);
  cudaFree(h->d_stage);
  cudaFree(h->d_dparam);
  cudaFree(h->d_pbar);
  cudaFree(h->d_tmax);
  cudaFree(h->ctape.pa);
  cudaFree(h->stape.pa);
  cudaFree(h->d_swork);
  cudaFree(h->d_sbnd);
  cudaFree(h->d_done);
  cudaFree(h->d_cellck);
  cudaFree(h->d_Y);
  for (auto& tri : h->ev)
    for (auto& e : tri)
      if (e) cudaEventDestroy(e);
  delete h;
  return NSW6_OK;
}

int nsw6_set_params(nsw6_handle* h, const nsw6_params* p) {
  if (!h || !p) return NSW6_ERR_BAD_ARG;
  h->params = *p;
  h->C = make_consts(h->params, h->opts);
  return NSW6_OK;
}

void nsw6_default_options(nsw6_options* o) {
  if (!o) return;
  o->roh2014 = 1;
  o->explicit_icegen = 1;
  o->kk2000 = 1;
  o->qi_sediment = 0;
  o->kin2kin = 0;
  o->aerosol_indirect = 0;
}

int nsw6_set_options(nsw6_handle* h, const nsw6_options* o) {
  if (!h || !o) return NSW6_ERR_BAD_ARG;
  const int v[6] = {o->roh2014, o->explicit_icegen, o->kk2000, o->qi_sediment, o->kin2kin, o->aerosol_indirect};
  for (int x : v)
    if (x != 0 && x != 1) return NSW6_ERR_BAD_ARG;
  h->opts = *o;
  h->opts.explicit_icegen = (o->roh2014 || o->explicit_icegen) ? 1 : 0;
  nsw6_options d;
  nsw6_default_options(&d);
  h->opt_active = std::memcmp(&h->opts, &d, sizeof(d)) != 0;
  h->C = make_consts(h->params, h->opts);
  return NSW6_OK;
}

int nsw6_get_options(const nsw6_handle* h, nsw6_options* o) {
  if (!h || !o) return NSW6_ERR_BAD_ARG;
  *o = h->opts;
  return NSW6_OK;
}

int nsw6_get_params(const nsw6_handle* h, nsw6_params* p) {
  if (!h || !p) return NSW6_ERR_BAD_ARG;
  *p = h->params;
  return NSW6_OK;
}

int nsw6_set_stream(nsw6_handle* h, void* stream) {
  if (!h) return NSW6_ERR_BAD_ARG;
  h->stream = (cudaStream_t)stream;
  return NSW6_OK;
}

int nsw6_set_sync_check(nsw6_handle* h, int sync_check) {
  if (!h) return NSW6_ERR_BAD_ARG;
  h->sync_check = sync_check;
  return NSW6_OK;
}

int nsw6_set_itelim(nsw6_handle* h, int itelim) {
  if (!h || itelim < 1) return NSW6_ERR_BAD_ARG;
  h->itelim = itelim;
  return NSW6_OK;
}

int nsw6_set_math(nsw6_handle* h, int mode) {
  if (!h || mode < 0 || mode > 1) return NSW6_ERR_BAD_ARG;
  h->math_lib = mode;
  return NSW6_OK;
}

int nsw6_set_adjoint_mode(nsw6_handle* h, int mode) {
  if (!h || mode < 0 || mode > 2) return NSW6_ERR_BAD_ARG;
  h->adj_mode = mode;
  return NSW6_OK;
}

int nsw6_set_precision(nsw6_handle* h, int mode) {
  if (!h || mode < 0 || mode > 2) return NSW6_ERR_BAD_ARG;
  h->mixed = mode;
  return NSW6_OK;
}

int nsw6_eval_math(nsw6_handle* h, int fn, const double* x, const double* y, double* out, int n) {
  if (!h || fn < 0 || fn > 2 || n < 0 || !x || !out || (fn == 2 && !y)) return NSW6_ERR_BAD_ARG;
  if (launch_math(fn, x, y, out, n, h->d_fmtab, h->stream) != cudaSuccess) return NSW6_ERR_CUDA;
  return cudaStreamSynchronize(h->stream) == cudaSuccess ? NSW6_OK : NSW6_ERR_CUDA;
}

int nsw6_set_timing(nsw6_handle* h, int on) {
  if (!h) return NSW6_ERR_BAD_ARG;
  h->timing = on;
  return NSW6_OK;
}

int nsw6_read_timing(nsw6_handle* h, double* t, int n, int* steps) {
  if (!h || !t || n < 2) return NSW6_ERR_BAD_ARG;
  const int rc = fold_timing(h);
  if (rc != NSW6_OK) return rc;
  t[0] = h->t_sum[0];
  t[1] = h->t_sum[1];
  if (steps) *steps = h->t_steps;
  h->t_sum[0] = h->t_sum[1] = 0.0;
  h->t_steps = 0;
  return NSW6_OK;
}

int nsw6_last_error(nsw6_handle* h, int* k, int* g, int* l, int* iters) {
  if (!h) return NSW6_ERR_BAD_ARG;
  DevStatus st;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return NSW6_ERR_CUDA;
  if (cudaMemcpy(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess) return NSW6_ERR_CUDA;
  if (st.code != 0 && cudaMemset(h->d_status, 0, sizeof(DevStatus)) != cudaSuccess) return NSW6_ERR_CUDA;
  if (k) *k = st.k;
  if (g) *g = st.g;
  if (l) *l = st.l;
  if (iters) *iters = st.iters;
  return st.code;
}

const char* nsw6_strerror(int status) {
  switch (status) {
    case NSW6_OK: return "success";
    case NSW6_ERR_BAD_ARG: return "bad argument";
    case NSW6_ERR_CUDA: return "CUDA runtime error";
    case NSW6_ERR_NOCONV: return "saturation adjustment did not converge";
    case NSW6_ERR_NAN: return "saturation adjustment produced a non-finite temperature";
    case NSW6_ERR_UNSUPPORTED: return "unsupported configuration";
    case NSW6_ERR_CHECK: return "adjoint self-check: the adjoint's forward differs from the step's";
    case NSW6_ERR_TOO_LARGE:
      return "region too large for mp_driver_noalloc (needs 5 <= kall <= 160 and gall * kall <= 2097152)";
    default: return "unknown status";
  }
}

int mp_driver(nsw6_handle* h, int l_region, double* rhog, double* rhogvx, double* rhogvy, double* rhogvz,
              double* rhogw, double* rhoge, double* rhogq, const double* vx, const double* vy, const double* vz,
              const double* w, const double* unccn, double* rho, double* tem, double* pre, double* q, double* qd,
              double* precip, double* ISO1_precip, double* ISO2_precip, double* precip_rhoe,
              double* precip_lh_heat, double* precip_rhophi, double* precip_rhokin, double* re_liquid,
              double* re_solid, double* re_cld, double* rctop, double* rwtop, double* tctop,
              const double* frhoge_af, const double* frhogqv_af, const double* frhoge_rad, const double* rhogqke,
              const double* gsgam2, const double* gsgam2h, const double* gam2, const double* gam2h,
              const double* ix, const double* iy, const double* iz, const double* jx, const double* jy,
              const double* jz, const double* z, const double* zh, double dt, double ct, double* GDCLW,
              double* GDCFRC, double* GPREC, const double* CBMFX) {
  (void)l_region;
  (void)ct;
  double* a[A_COUNT] = {rhog, rhogvx, rhogvy, rhogvz, rhogw, rhoge, rhogq,
                        (double*)vx, (double*)vy, (double*)vz, (double*)w, (double*)unccn,
                        rho, tem, pre, q, qd, precip, ISO1_precip, ISO2_precip,
                        precip_rhoe, precip_lh_heat, precip_rhophi, precip_rhokin,
                        re_liquid, re_solid, re_cld, rctop, rwtop, tctop,
                        (double*)frhoge_af, (double*)frhogqv_af, (double*)frhoge_rad, (double*)rhogqke,
                        (double*)gsgam2, (double*)gsgam2h, (double*)gam2, (double*)gam2h,
                        (double*)ix, (double*)iy, (double*)iz, (double*)jx, (double*)jy, (double*)jz,
                        (double*)z, (double*)zh, GDCLW, GDCFRC, GPREC, (double*)CBMFX};
  if (!h) return NSW6_ERR_BAD_ARG;
  h->region_call = 1;
  const int rc = run(h, 1, a, dt);
  h->region_call = 0;
  return rc;
}

int nsw6_set_precip_stride(nsw6_handle* h, long long ld) {
  if (!h || ld < 0 || (ld > 0 && ld < h->gall)) return NSW6_ERR_BAD_ARG;
  h->prec_ld = ld;
  return NSW6_OK;
}

int mp_driver_mixed(nsw6_handle* h, int l_region, double* rhog, double* rhogvx, double* rhogvy, double* rhogvz,
                    double* rhogw, double* rhoge, double* rhogq, const double* vx, const double* vy,
                    const double* vz, const double* w, const double* unccn, double* rho, double* tem, double* pre,
                    double* q, double* qd, double* precip, double* ISO1_precip, double* ISO2_precip,
                    double* precip_rhoe, double* precip_lh_heat, double* precip_rhophi, double* precip_rhokin,
                    double* re_liquid, double* re_solid, double* re_cld, double* rctop, double* rwtop,
                    double* tctop, const double* frhoge_af, const double* frhogqv_af, const double* frhoge_rad,
                    const double* rhogqke, const double* gsgam2, const double* gsgam2h, const double* gam2,
                    const double* gam2h, const double* ix, const double* iy, const double* iz, const double* jx,
                    const double* jy, const double* jz, const double* z, const double* zh, double dt, double ct,
                    double* GDCLW, double* GDCFRC, double* GPREC, const double* CBMFX) {
  if (!h) return NSW6_ERR_BAD_ARG;
  const int saved = h->mixed;
  h->mixed = 1;
  const int rc = mp_driver(h, l_region, rhog, rhogvx, rhogvy, rhogvz, rhogw, rhoge, rhogq, vx, vy, vz, w, unccn,
                           rho, tem, pre, q, qd, precip, ISO1_precip, ISO2_precip, precip_rhoe, precip_lh_heat,
                           precip_rhophi, precip_rhokin, re_liquid, re_solid, re_cld, rctop, rwtop, tctop,
                           frhoge_af, frhogqv_af, frhoge_rad, rhogqke, gsgam2, gsgam2h, gam2, gam2h, ix, iy, iz,
                           jx, jy, jz, z, zh, dt, ct, GDCLW, GDCFRC, GPREC, CBMFX);
  h->mixed = saved;
  return rc;
}

int mp_driver_batched(nsw6_handle* h, int lall, double* rhog, double* rhogvx, double* rhogvy, double* rhogvz,
                      double* rhogw, double* rhoge, double* rhogq, const double* vx, const double* vy,
                      const double* vz, const double* w, const double* unccn, double* rho, double* tem, double* pre,
                      double* q, double* qd, double* precip, double* ISO1_precip, double* ISO2_precip,
                      double* precip_rhoe, double* precip_lh_heat, double* precip_rhophi, double* precip_rhokin,
                      double* re_liquid, double* re_solid, double* re_cld, double* rctop, double* rwtop,
                      double* tctop, const double* frhoge_af, const double* frhogqv_af, const double* frhoge_rad,
                      const double* rhogqke, const double* gsgam2, const double* gsgam2h, const double* gam2,
                      const double* gam2h, const double* ix, const double* iy, const double* iz, const double* jx,
                      const double* jy, const double* jz, const double* z, const double* zh, double dt, double ct,
                      double* GDCLW, double* GDCFRC, double* GPREC, const double* CBMFX) {
  (void)ct;
  double* a[A_COUNT] = {rhog, rhogvx, rhogvy, rhogvz, rhogw, rhoge, rhogq,
                        (double*)vx, (double*)vy, (double*)vz, (double*)w, (double*)unccn,
                        rho, tem, pre, q, qd, precip, ISO1_precip, ISO2_precip,
                        precip_rhoe, precip_lh_heat, precip_rhophi, precip_rhokin,
                        re_liquid, re_solid, re_cld, rctop, rwtop, tctop,
                        (double*)frhoge_af, (double*)frhogqv_af, (double*)frhoge_rad, (double*)rhogqke,
                        (double*)gsgam2, (double*)gsgam2h, (double*)gam2, (double*)gam2h,
                        (double*)ix, (double*)iy, (double*)iz, (double*)jx, (double*)jy, (double*)jz,
                        (double*)z, (double*)zh, GDCLW, GDCFRC, GPREC, (double*)CBMFX};
  return run(h, lall, a, dt);
}

int mp_driver_argv(nsw6_handle* h, int lall, double* const* args, double dt, double ct, int host) {
  (void)ct;
  if (!h || !args || lall < 1 || lall > h->lall_max) return NSW6_ERR_BAD_ARG;
  if (!host) return run(h, lall, args, dt);
  return run_host(h, lall, args, dt);
}

int nsw6_host_copy_bytes(const nsw6_handle* h, int lall, unsigned long long* h2d, unsigned long long* d2h) {
  if (!h || lall < 1 || lall > h->lall_max) return NSW6_ERR_BAD_ARG;
  unsigned long long in = 0, out = 0;
  for (int i = 0; i < A_COUNT; ++i) {
    in += sizeof(double) * host_in_doubles(h, i, lall);
    if (arg_is_written(i)) out += sizeof(double) * arg_region_elems(i, h->kall, h->gall) * (size_t)lall;
  }
  if (h2d) *h2d = in;
  if (d2h) *d2h = out;
  return NSW6_OK;
}

int mp_driver_steps(nsw6_handle* h, int lall, double* const* args, double dt, double ct, int nsteps) {
  (void)ct;
  if (!h || !args || lall < 1 || lall > h->lall_max || nsteps < 0) return NSW6_ERR_BAD_ARG;
  if (h->mixed == 2) {   // the serial-column check path: plain calls
    for (int i = 0; i < nsteps; ++i) {
      const int rc = run(h, lall, args, dt);
      if (rc != NSW6_OK) return rc;
    }
    return NSW6_OK;
  }
  Problem P;
  int rc = fill_problem(h, lall, args, dt, P);
  if (rc != NSW6_OK) return rc;
  bool same = h->graph && h->graph_lall == lall && h->graph_dt == dt && h->graph_mixed == h->mixed &&
              h->graph_math == h->math_lib && h->graph_itelim == h->itelim &&
              std::memcmp(&h->graph_params, &h->params, sizeof(nsw6_params)) == 0 &&
              std::memcmp(&h->graph_opts, &h->opts, sizeof(nsw6_options)) == 0;
  for (int i = 0; same && i < A_COUNT; ++i) same = h->graph_args[i] == args[i];
  if (!same) {
    if (h->graph) {
      cudaGraphExecDestroy(h->graph);
      h->graph = nullptr;
    }
    if (!h->cap_stream && cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
      return NSW6_ERR_CUDA;
    if (launch_prepare() != cudaSuccess) return NSW6_ERR_CUDA;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return NSW6_ERR_CUDA;
    const cudaError_t le = launch_step(P, h->C, h->cap_stream, nullptr);
    const cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess || !g) {
      if (g) cudaGraphDestroy(g);
      return NSW6_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      h->graph = nullptr;
      return NSW6_ERR_CUDA;
    }
    for (int i = 0; i < A_COUNT; ++i) h->graph_args[i] = args[i];
    h->graph_lall = lall;
    h->graph_dt = dt;
    h->graph_mixed = h->mixed;
    h->graph_math = h->math_lib;
    h->graph_itelim = h->itelim;
    h->graph_params = h->params;
    h->graph_opts = h->opts;
  }
  for (int i = 0; i < nsteps; ++i)
    if (cudaGraphLaunch(h->graph, h->stream) != cudaSuccess) return NSW6_ERR_CUDA;
  return finish(h, cudaSuccess);
}

int mp_driver_tlm(nsw6_handle* h, int lall, double* const* args, double* const* targs, const double* dparams,
                  double dt, double ct) {
  (void)ct;
  // adjoint mode 1: the serial column step over Dual (one column per thread);
  // otherwise the stages in forward mode, every cell in parallel
  const bool serial = h && h->adj_mode == 1;
  int rc = deriv_check(h, lall, args, targs, serial);
  if (rc != NSW6_OK) return rc;
  if (serial && (rc = deriv_prepass(h, lall, args, dt)) != NSW6_OK) return rc;
  Problem P;
  rc = fill_problem(h, lall, args, dt, P);
  if (rc != NSW6_OK) return rc;
  double hp[16] = {};
  std::memcpy(hp, &h->params, sizeof(double) * 7);
  if (dparams) std::memcpy(hp + 8, dparams, sizeof(double) * 7);
  if (cudaMemcpyAsync(h->d_dparam, hp, sizeof(hp), cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    return NSW6_ERR_CUDA;
  ArgPtrs x, dx;
  for (int i = 0; i < A_COUNT; ++i) {
    x.a[i] = args[i];
    dx.a[i] = targs[i];
  }
  if (serial) {
    rc = finish(h, launch_tlm(P, h->C, x, dx, h->d_dparam, h->d_dparam + 8, h->stream));
  } else {
    if ((rc = ensure_adj_work(h)) != NSW6_OK) return rc;
    rc = finish(h, launch_tlm_staged(P, h->C, x, dx, h->d_dparam, h->d_dparam + 8, h->d_Y, h->d_swork, h->d_sbnd,
                                     h->stream));
  }
  if (!h->sync_check && rc == NSW6_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) return NSW6_ERR_CUDA;
  return rc;
}

// (Re)allocates a set of interleaved tapes: nslot threads x cap entries.
int ensure_tape(TapeMem& t, size_t& bytes, int nslot, int cap) {
  const size_t per = sizeof(int) * 2 + sizeof(double) * 3;
  const size_t need = per * (size_t)cap * (size_t)nslot;
  if (t.pa && need <= bytes && t.nslot == nslot && t.cap >= cap) return NSW6_OK;
  cudaFree(t.pa);
  t = TapeMem{};
  bytes = 0;
  char* base = nullptr;
  if (cudaMalloc(&base, need) != cudaSuccess) return NSW6_ERR_CUDA;
  const size_t n = (size_t)cap * nslot;
  t.pa = reinterpret_cast<int*>(base);
  t.pb = t.pa + n;
  t.da = reinterpret_cast<double*>(base + sizeof(int) * 2 * n);
  t.db = t.da + n;
  t.adj = t.db + n;
  t.nslot = nslot;
  t.cap = cap;
  bytes = need;
  return NSW6_OK;
}

int mp_driver_adjoint(nsw6_handle* h, int lall, double* const* args, double* const* aargs, double* dparams,
                      double dt, double ct) {
  (void)ct;
  int rc = deriv_check(h, lall, args, aargs, false);
  if (rc != NSW6_OK) return rc;
  Problem P;
  rc = fill_problem(h, lall, args, dt, P);
  if (rc != NSW6_OK) return rc;
  if (cudaMemcpyAsync(h->d_dparam, &h->params, sizeof(double) * 7, cudaMemcpyHostToDevice, h->stream) !=
      cudaSuccess)
    return NSW6_ERR_CUDA;
  ArgPtrs x, xb;
  for (int i = 0; i < A_COUNT; ++i) {
    x.a[i] = args[i];
    xb.a[i] = aargs[i];
  }
  if ((rc = ensure_adj_work(h)) != NSW6_OK) return rc;
  // the all-regions layout of Y for this call's lall
  const size_t NCl = (size_t)lall * h->kall * h->gall;
  double* Y = h->d_Y;
  double* YB = h->d_Y + (size_t)adj_nfields() * NCl;
  auto round_slots = [](long long n, int maxs) {
    long long s = ((n + DERIV_THREADS - 1) / DERIV_THREADS) * DERIV_THREADS;
    return (int)(s > maxs ? maxs : s);
  };
  const long long ncell = (long long)lall * (h->kall - 2) * h->gall;
  const int ncell_slots = round_slots(ncell, ADJ_CELL_SLOTS);
  // the stage tapes serve the recorded form (adj_mode 1), and S4 with the
  // mixed-phase saturation adjustment or KIN2KIN
  if ((h->adj_mode == 1 || (h->opt_active && (!h->opts.explicit_icegen || h->opts.kin2kin))) &&
      (rc = ensure_tape(h->stape, h->stape_bytes, adj_stage_slots(), adj_stage_tape_cap())) != NSW6_OK)
    return rc;
  h->stape.count_only = 0;
  double pb[8] = {};
  // the cell phase's outputs, then the column phase's adjoint (level-parallel stages)
  // the cell phase: hand-written, or recorded (adj_mode 1, and with the scheme
  // switches, whose cell physics the hand-written sweep does not cover)
  const bool recorded = h->adj_mode == 1 || h->opt_active;
  // with the mixed-precision step selected, the hand-written adjoint
  // linearises that step: its cell physics (FP32 rates, FP64 budgets) and its
  // FP32 departure distances
  const int mixed_cell = (h->mixed == 1 && !recorded) ? 1 : 0;
  if (!recorded && !h->d_cellck &&
      cudaMalloc(&h->d_cellck, sizeof(double) * adj_cell_ck_doubles(h->lall_max, h->kall, h->gall)) != cudaSuccess)
    return NSW6_ERR_CUDA;
  if ((recorded ? launch_adj_cellfwd(P, h->C, x, Y, h->stream)
                : launch_adj_cell_save(P, h->C, x, Y, h->d_cellck, h->adj_mode == 2, mixed_cell, h->stream)) !=
          cudaSuccess ||
      launch_adj_column_staged(P, h->C, x, xb, Y, YB, adj_nfields(), h->d_swork, h->d_sbnd, h->stape, h->adj_mode == 1,
                               mixed_cell, h->stream) != cudaSuccess ||
      cudaMemsetAsync(h->d_pbar, 0, sizeof(double) * 8, h->stream) != cudaSuccess ||
      (recorded && cudaMemsetAsync(h->d_done, 0, sizeof(int) * (size_t)ncell, h->stream) != cudaSuccess))
    return NSW6_ERR_CUDA;
  // the cell phase's adjoint: hand-written, or (adj_mode 1) recorded on a tape
  // as long as the longest cell's record (measured once, then kept; a longer
  // record makes the launch repeat for the cells that did not fit)
  if (!recorded) {
    if (launch_adj_cell_hw(P, h->C, x, xb, YB, h->d_pbar, h->d_cellck, mixed_cell, h->stream) != cudaSuccess)
      return NSW6_ERR_CUDA;
  } else {
    for (int attempt = 0; attempt < 3; ++attempt) {
      if (!h->ctape.pa || attempt > 0) {
        int tcell = 0;
        TapeMem cnt{};
        cnt.count_only = 1;
        cnt.nslot = ncell_slots;
        if (cudaMemsetAsync(h->d_tmax, 0, sizeof(int), h->stream) != cudaSuccess ||
            launch_adj_cell(P, h->C, x, xb, YB, cnt, h->d_dparam, h->d_pbar, h->d_tmax, h->d_done, h->stream) !=
                cudaSuccess ||
            cudaMemcpyAsync(&tcell, h->d_tmax, sizeof(int), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess)
          return NSW6_ERR_CUDA;
        if ((rc = ensure_tape(h->ctape, h->ctape_bytes, ncell_slots, tcell + tcell / 4 + 64)) != NSW6_OK) return rc;
      }
      h->ctape.count_only = 0;
      if (h->ctape.nslot != ncell_slots &&
          (rc = ensure_tape(h->ctape, h->ctape_bytes, ncell_slots, h->ctape.cap)) != NSW6_OK)
        return rc;
      int t2 = 0;
      if (cudaMemsetAsync(h->d_tmax, 0, sizeof(int), h->stream) != cudaSuccess ||
          launch_adj_cell(P, h->C, x, xb, YB, h->ctape, h->d_dparam, h->d_pbar, h->d_tmax, h->d_done, h->stream) !=
              cudaSuccess ||
          cudaMemcpyAsync(&t2, h->d_tmax, sizeof(int), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
          cudaStreamSynchronize(h->stream) != cudaSuccess)
        return NSW6_ERR_CUDA;
      if (t2 <= h->ctape.cap) break;
      if (attempt == 2) return NSW6_ERR_UNSUPPORTED;
    }
  }
  if (cudaMemcpyAsync(pb, h->d_pbar, sizeof(double) * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return NSW6_ERR_CUDA;
  if (dparams)
    for (int i = 0; i < 7; ++i) dparams[i] += pb[i];
  return nsw6_last_error(h, nullptr, nullptr, nullptr, nullptr);
}

}  // extern "C"

// ------------------------------------------------------- mp_driver_noalloc
// Fixed scratch of mp_driver_noalloc, in doubles; every slot starts on a
// 256-byte boundary.  The departure distances take 6 doubles per cell.
namespace {
constexpr size_t NA_STATUS = 0;                                   // DevStatus (256 B slot)
constexpr size_t NA_ZMAX = NA_STATUS + 32;                        // [6][MAX_KALL] uint64 keys
constexpr size_t NA_ZMIN = NA_ZMAX + 6 * MAX_KALL;                // [6][MAX_KALL] uint64 keys
constexpr size_t NA_GRID = NA_ZMIN + 6 * MAX_KALL;                // [GF_COUNT][MAX_KALL]
constexpr size_t NA_FMTAB = NA_GRID + (size_t)GF_COUNT * MAX_KALL; // [FM_TABLE_DOUBLES]
constexpr size_t NA_ZDIS = ((NA_FMTAB + FM_TABLE_DOUBLES + 31) / 32) * 32;  // [6][kall][gall]
constexpr size_t NA_SATQ = NA_ZDIS + 6 * (size_t)NSW6_NOALLOC_MAX_CELLS;  // [1 + cells] uint32
constexpr size_t NA_TOTAL = NA_SATQ + ((size_t)NSW6_NOALLOC_MAX_CELLS + 2) / 2;
static_assert(NA_ZMAX % 32 == 0 && NA_ZMIN % 32 == 0 && NA_GRID % 32 == 0 && NA_FMTAB % 32 == 0,
              "scratch slots must stay 256-byte aligned");
static_assert(sizeof(DevStatus) <= 32 * sizeof(double), "status slot too small");

static __device__ __align__(256) double g_noalloc_scratch[NA_TOTAL];

// Device address of the scratch on the current device.  Looked up on every
// call (cheap once the module is loaded) rather than cached, so that a device
// reset or a new context between calls cannot leave a stale address.
int noalloc_scratch(double** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return NSW6_ERR_CUDA;
  *out = static_cast<double*>(p);
  return NSW6_OK;
}
}  // namespace

extern "C" int mp_driver_noalloc(int gall, int kall, const double* gz, const double* gzh,
                                 const nsw6_params* params, double* const* args, double dt, double ct,
                                 void* stream) {
  (void)ct;
  if (!gz || !gzh || !args) return NSW6_ERR_BAD_ARG;
  if (gall < 1 || kall < 5) return NSW6_ERR_BAD_ARG;
  if (kall > MAX_KALL || (long long)gall * kall > NSW6_NOALLOC_MAX_CELLS) return NSW6_ERR_TOO_LARGE;
  // The call ends with a synchronising read of the status word, which a
  // capturing stream does not allow: refuse before issuing anything.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess) return NSW6_ERR_CUDA;
  if (cap != cudaStreamCaptureStatusNone) return NSW6_ERR_UNSUPPORTED;
  double* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc != NSW6_OK) return rc;

  // A handle on the stack whose workspace pointers are slots of the scratch.
  nsw6_handle h;
  h.gall = gall;
  h.kall = kall;
  h.lall_max = 1;
  if (params) h.params = *params;
  else nsw6_default_params(&h.params);
  h.C = make_consts(h.params);
  h.d_grid = base + NA_GRID;
  h.d_fmtab = base + NA_FMTAB;
  h.d_zdis = base + NA_ZDIS;
  h.d_zmax = reinterpret_cast<unsigned long long*>(base + NA_ZMAX);
  h.d_zmin = reinterpret_cast<unsigned long long*>(base + NA_ZMIN);
  h.d_satq = reinterpret_cast<unsigned*>(base + NA_SATQ);
  h.d_status = reinterpret_cast<DevStatus*>(base + NA_STATUS);
  h.stream = static_cast<cudaStream_t>(stream);

  Problem P;
  rc = fill_problem(&h, 1, args, dt, P);
  if (rc != NSW6_OK) return rc;

  // Grid metrics and fast-math tables, computed on the host stack and copied
  // into the scratch (pageable source: the copy has consumed it on return).
  double hbuf[GF_COUNT * MAX_KALL + FM_TABLE_DOUBLES];
  make_grid(kall, gz, gzh, hbuf);
  build_fastmath_tables(hbuf + GF_COUNT * MAX_KALL);
  if (cudaMemcpyAsync(h.d_grid, hbuf, sizeof(double) * GF_COUNT * (size_t)kall, cudaMemcpyHostToDevice,
                      h.stream) != cudaSuccess ||
      cudaMemcpyAsync(h.d_fmtab, hbuf + GF_COUNT * MAX_KALL, sizeof(double) * FM_TABLE_DOUBLES,
                      cudaMemcpyHostToDevice, h.stream) != cudaSuccess ||
      cudaMemsetAsync(h.d_status, 0, sizeof(DevStatus), h.stream) != cudaSuccess)
    return NSW6_ERR_CUDA;
  if (launch_step(P, h.C, h.stream, nullptr) != cudaSuccess) return NSW6_ERR_CUDA;
  DevStatus st;
  if (cudaMemcpyAsync(&st, h.d_status, sizeof(st), cudaMemcpyDeviceToHost, h.stream) != cudaSuccess ||
      cudaStreamSynchronize(h.stream) != cudaSuccess)
    return NSW6_ERR_CUDA;
  return st.code;
}
