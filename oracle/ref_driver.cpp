// Oracle driver for the reference NSW6 sources (TEST INFRASTRUCTURE ONLY).
//
// It replaces the reference's main.cpp (src/main.cpp:14-372): instead of
// reading snapshot files it exposes a C entry point that wraps caller arrays
// in (shim) Kokkos views and calls the reference's own, unmodified
// MP_DRIVER::mp_driver (src/mod_mp_driver.cpp:335-613) on one region.
// The set-up sequence mirrors main.cpp:177-189: GRD_Setup, CVW_CPW_Setup,
// SATURATION_Setup, mp_init("NSW6").
//
// Compiled together with a copy of the reference sources whose compile-time
// sizes (include/problemsize.h:62-79) were patched by oracle/build_ref.py.
#include <sys/stat.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#include "problemsize.h"
#include "data_io.h"
#include "mod_debug.h"
#include "mod_satadjust.h"
#include "mod_mp_driver.h"

using namespace PROBLEM_SIZE;

#ifdef NSW6REF_OPTIONS
// Scheme switches of the "opt" build (oracle/build_ref.py): the two choices
// mp_nsw6_init assigns from literals read these variables instead, and the
// others are the reference's own globals (src/mod_mp_nsw6.cpp:127-132,
// src/problemsize.cpp:39).
bool nsw6ref_opt_roh = true;
bool nsw6ref_opt_kk2000 = true;
extern std::string precip_transport_type;
extern bool OPT_EXPLICIT_ICEGEN;
extern bool OPT_INDIR;
#endif

namespace {

struct CoutSilencer {
  std::streambuf* old = nullptr;
  std::ostringstream sink;
  explicit CoutSilencer(bool on) {
    if (on) old = std::cout.rdbuf(sink.rdbuf());
  }
  ~CoutSilencer() {
    if (old) std::cout.rdbuf(old);
  }
};

bool g_ready = false;
bool g_quiet = true;

bool write_raw(const std::string& path, const double* v, size_t n) {
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  f.write(reinterpret_cast<const char*>(v), std::streamsize(n * sizeof(double)));
  return bool(f);
}

}  // namespace

extern "C" {

int nsw6ref_gall() { return int(ADM_gall_in); }
int nsw6ref_kall() { return int(ADM_kall); }
int nsw6ref_kmin() { return int(kmin); }
int nsw6ref_kmax() { return int(kmax); }
int nsw6ref_abort_count() { return Kokkos::shim::abort_count().load(); }
void nsw6ref_set_quiet(int q) { g_quiet = (q != 0); }

// Grid/constant set-up.  GRD_Input_vgrid (mod_debug.cpp:189-195) reads
// "data/vgrid/GRD_{gz,gzh}.dat" relative to the working directory, so the
// interface heights are written in the reference's raw FP64 format into a
// scratch directory that is made current for the duration of the call.
int nsw6ref_setup(const double* gz, const double* gzh) {
  CoutSilencer quiet(g_quiet);
  char tmpl[] = "/tmp/nsw6ref_XXXXXX";
  char* dir = mkdtemp(tmpl);
  if (!dir) return 1;
  std::string d(dir);
  mkdir((d + "/data").c_str(), 0700);
  mkdir((d + "/data/vgrid").c_str(), 0700);
  if (!write_raw(d + "/data/vgrid/GRD_gz.dat", gz, ADM_kall)) return 2;
  if (!write_raw(d + "/data/vgrid/GRD_gzh.dat", gzh, ADM_kall)) return 3;

  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return 4;
  if (chdir(d.c_str()) != 0) return 5;

  GRD_gz = View1D<double, DEFAULT_MEM>("GRD_gz   ", ADM_kall);
  GRD_gzh = View1D<double, DEFAULT_MEM>("GRD_gzh  ", ADM_kall);
  GRD_dgz = View1D<double, DEFAULT_MEM>("GRD_dgz  ", ADM_kall);
  GRD_dgzh = View1D<double, DEFAULT_MEM>("GRD_dgzh ", ADM_kall);
  GRD_rdgz = View1D<double, DEFAULT_MEM>("GRD_rdgz ", ADM_kall);
  GRD_rdgzh = View1D<double, DEFAULT_MEM>("GRD_rdgzh", ADM_kall);
  GRD_afact = View1D<double, DEFAULT_MEM>("GRD_afact", ADM_kall);
  GRD_bfact = View1D<double, DEFAULT_MEM>("GRD_bfact", ADM_kall);
  GRD_cfact = View1D<double, DEFAULT_MEM>("GRD_cfact", ADM_kall);
  GRD_dfact = View1D<double, DEFAULT_MEM>("GRD_dfact", ADM_kall);
  CVW = View1D<double, DEFAULT_MEM>("CVW", 6);
  CPW = View1D<double, DEFAULT_MEM>("CPW", 6);

  DEBUG::GRD_Setup();
  DEBUG::CVW_CPW_Setup();
  SATADJUST::SATURATION_Setup();
  // mp_nsw6_init assigns some members of the global para only in its
  // Roh_flag branch (mod_mp_nsw6.cpp:345-357); start from the GlobalParams
  // defaults, as a fresh process does, so that a set-up does not inherit the
  // values of an earlier one.
  para = GlobalParams();
  MP_DRIVER::mp_init(MP_TYPE);

  int rc = chdir(cwd);
  std::remove((d + "/data/vgrid/GRD_gz.dat").c_str());
  std::remove((d + "/data/vgrid/GRD_gzh.dat").c_str());
  rmdir((d + "/data/vgrid").c_str());
  rmdir((d + "/data").c_str());
  rmdir(d.c_str());
  g_ready = true;
  return rc == 0 ? 0 : 6;
}

// Overrides of the tunable scheme parameters held in the reference's global
// GlobalParams (mod_mp_nsw6.h:16-123), applied after mp_init:
//   p[0] beta_saut, p[1] qicrt_saut, p[2] Cr, p[3] Cs, p[4] Cg.
// The KK2000 autoconversion rate (mod_mp_nsw6.cpp:1154) and the ice
// nucleation coefficient (mod_mp_nsw6.cpp:1083) are literals in the reference
// and cannot be changed here.
int nsw6ref_set_params(const double* p) {
  if (!g_ready) return 1;
  para.beta_saut = p[0];
  para.qicrt_saut = p[1];
  para.Cr = p[2];
  para.Cs = p[3];
  para.Cg = p[4];
  return 0;
}

// Scheme switches (the "opt" build only; they take effect at the next
// nsw6ref_setup, whose mp_init runs mp_nsw6_init):
//   o[0] Roh_flag (Roh and Satoh 2014 snow settings, mod_mp_nsw6.cpp:345-357)
//   o[1] OPT_EXPLICIT_ICEGEN (mp_nsw6_init forces it on when Roh_flag is set)
//   o[2] KK2000 warm rain (1) or Berry (0), mod_mp_nsw6.cpp:374-387
//   o[3] precip_transport_type "4WATER" (1) or "3WATER" (0)
//   o[4] PRCIP_TRN_ECORRECT "KIN2KIN" (1) or "KIN2EIN" (0)
//   o[5] OPT_INDIR (cloud number from unccn)
// Returns 1 in builds without the switches.
int nsw6ref_set_options(const int* o) {
#ifdef NSW6REF_OPTIONS
  nsw6ref_opt_roh = o[0] != 0;
  OPT_EXPLICIT_ICEGEN = o[1] != 0;
  nsw6ref_opt_kk2000 = o[2] != 0;
  precip_transport_type = o[3] ? "4WATER" : "3WATER";
  PRCIP_TRN_ECORRECT = o[4] ? "KIN2KIN" : "KIN2EIN";
  OPT_INDIR = o[5] != 0;
  return 0;
#else
  (void)o;
  return 1;
#endif
}

int nsw6ref_get_params(double* p) {
  p[0] = para.beta_saut;
  p[1] = para.qicrt_saut;
  p[2] = para.Cr;
  p[3] = para.Cs;
  p[4] = para.Cg;
  return 0;
}

// One call of the reference mp_driver on one region.  `a` holds the 50 array
// arguments of mp_driver in the reference's order (mod_mp_driver.h:71-124):
// 2-D fields [kall][gall], tracers [6][kall][gall], precip-type fields
// [2][gall], column fields [gall] or [1][gall].  All are contiguous.
// Returns 0, or 10 + n when the shim recorded n device aborts (satadjust
// Newton non-convergence).
int nsw6ref_mp_driver(int l_region, double* const* a, double dt, double ct) {
  if (!g_ready) return 1;
  CoutSilencer quiet(g_quiet);
  const size_t K = ADM_kall, G = ADM_gall_in, NQ = nqmax;
  auto v2 = [&](int i) { return View2D<double, DEFAULT_MEM>(a[i], K, G); };
  auto v3 = [&](int i) { return View3D<double, DEFAULT_MEM>(a[i], NQ, K, G); };
  auto p2 = [&](int i) { return View2D<double, DEFAULT_MEM>(a[i], size_t(2), G); };
  auto c1 = [&](int i) { return View1D<double, DEFAULT_MEM>(a[i], G); };
  auto t2 = [&](int i) { return View2D<double, DEFAULT_MEM>(a[i], size_t(1), G); };

  const int before = Kokkos::shim::abort_count().load();
  MP_DRIVER::mp_driver(l_region,
                       v2(0), v2(1), v2(2), v2(3), v2(4), v2(5),  // rhog .. rhoge
                       v3(6),                                     // rhogq
                       v2(7), v2(8), v2(9), v2(10), v2(11),       // vx vy vz w unccn
                       v2(12), v2(13), v2(14),                    // rho tem pre
                       v3(15),                                    // q
                       v2(16),                                    // qd
                       p2(17), p2(18), p2(19),                    // precip, ISO1, ISO2
                       c1(20), c1(21), c1(22), c1(23),            // precip_rhoe .. rhokin
                       v2(24), v2(25), v2(26),                    // re_liquid re_solid re_cld
                       t2(27), t2(28), t2(29),                    // rctop rwtop tctop
                       v2(30), v2(31), v2(32), v2(33),            // frhoge_af .. rhogqke
                       v2(34), v2(35), v2(36), v2(37),            // gsgam2 gsgam2h gam2 gam2h
                       c1(38), c1(39), c1(40), c1(41), c1(42), c1(43),  // ix .. jz
                       v2(44), v2(45),                            // z zh
                       dt, ct,
                       v2(46), v2(47), v2(48), v2(49));           // GDCLW GDCFRC GPREC CBMFX
  const int n = Kokkos::shim::abort_count().load() - before;
  return n == 0 ? 0 : 10 + n;
}

// The reference's own snapshot readers (src/data_io.cpp), for checking the
// package's snapshot module against them: out receives the file's contents in
// the harness's array layout (ADM_lall = 1 in these builds).
void nsw6ref_read_1d(const char* fname, double* out) {
  DATA_IO::read_data_1d(fname, out);
}
void nsw6ref_read_2d(const char* fname, double* out) {
  DATA_IO::read_data_2d(fname, reinterpret_cast<double(*)[ADM_gall_in]>(out));
}
void nsw6ref_read_3d(const char* fname, double* out) {
  DATA_IO::read_data_3d(fname, reinterpret_cast<double(*)[ADM_kall][ADM_gall_in]>(out));
}
void nsw6ref_read_4d(const char* fname, double* out) {
  DATA_IO::read_data_4d(fname, reinterpret_cast<double(*)[TRC_VMAX][ADM_kall][ADM_gall_in]>(out));
}
void nsw6ref_read_precip(const char* fname, double* out) {
  DATA_IO::read_data_4d(fname, reinterpret_cast<double(*)[ADM_lall][ADM_KNONE][ADM_gall_in]>(out));
}

}  // extern "C"
