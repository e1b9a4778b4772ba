/* nsw6.h - C ABI of the GB300-native NICAM NSW6 microphysics step.
 *
 * Drop-in for the reference's MP_DRIVER::mp_driver (Kokkos version,
 * src/mod_mp_driver.h:71-124, src/mod_mp_driver.cpp:335-613) with
 * MP_TYPE = "NSW6": same argument list, same order, same (gall, kall, lall)
 * structure-of-arrays layout (C order, g fastest), FP64, updated in place.
 * Pointers are CUDA device pointers unless a function says otherwise.
 *
 * The one-time set-up the reference performs through process globals
 * (GRD_Setup mod_debug.cpp:92-187, CVW_CPW_Setup mod_debug.cpp:76-90,
 * SATURATION_Setup mod_satadjust.cpp:24-47, mp_init/mp_nsw6_init
 * mod_mp_driver.cpp:11-24 / mod_mp_nsw6.cpp:276-434) is held in an opaque
 * handle instead, so several grids can coexist in one process.
 *
 * Error convention: every function returns an nsw6_status (0 = success).
 * The device never traps: a saturation-adjustment Newton iteration that does
 * not converge (the reference calls Kokkos::abort, mod_satadjust.cpp:883-891)
 * is recorded in a device status word and reported as NSW6_ERR_NOCONV or
 * NSW6_ERR_NAN; nsw6_last_error() gives the first failing cell.
 *
 * Threading: a handle is not re-entrant; calls on one handle must not overlap.
 * All work of a call is issued on the handle's CUDA stream.
 */
#ifndef NSW6_H
#define NSW6_H

#ifdef __cplusplus
extern "C" {
#endif

#define NSW6_ABI_VERSION 1

typedef enum nsw6_status {
  NSW6_OK = 0,
  NSW6_ERR_BAD_ARG = 1,      /* null pointer, bad size, region out of range          */
  NSW6_ERR_CUDA = 2,         /* a CUDA runtime call failed                           */
  NSW6_ERR_NOCONV = 3,       /* satadjust Newton hit the iteration limit             */
  NSW6_ERR_NAN = 4,          /* satadjust produced a non-finite temperature          */
  NSW6_ERR_UNSUPPORTED = 5,  /* configuration not implemented                        */
  NSW6_ERR_TOO_LARGE = 6,    /* region larger than mp_driver_noalloc's fixed scratch,
                                or gall kall lall_max >= 2^32 at nsw6_create          */
  NSW6_ERR_CHECK = 7         /* adjoint mode 2: its forward differs from the step's  */
} nsw6_status;

/* Tunable NSW6 scheme parameters (GlobalParams, src/mod_mp_nsw6.h:16-123,
 * values as set by mp_nsw6_init).  Differentiable parameters of the
 * tangent-linear/adjoint entry points follow this order. */
typedef struct nsw6_params {
  double beta_saut;   /* ice->snow autoconversion rate      [1/s]  mod_mp_nsw6.cpp:287-294, used :1162 */
  double qicrt_saut;  /* ice->snow autoconversion threshold [kg/kg] mod_mp_nsw6.h:87, used :1163       */
  double Cr;          /* rain fall-speed coefficient               mod_mp_nsw6.h:27, used :1076         */
  double Cs;          /* snow fall-speed coefficient               mod_mp_nsw6.h:28, used :1077         */
  double Cg;          /* graupel fall-speed coefficient            mod_mp_nsw6.cpp:337, used :1078      */
  double ice_nuc;     /* ice nucleation coefficient of Qi0         literal at mod_mp_nsw6.cpp:1083      */
  double kk_aut;      /* KK2000 warm-rain autoconversion rate      literal at mod_mp_nsw6.cpp:1156      */
} nsw6_params;

typedef struct nsw6_handle nsw6_handle;

/* Fills *p with the values of the reference configuration. */
void nsw6_default_params(nsw6_params* p);

/* Creates a handle for regions of gall columns and kall levels (5 <= kall <=
 * 160; kmin = 1, kmax = kall-2, as include/problemsize.h:62-79) and up to lall_max regions
 * per batched call.  gz/gzh are the full-level and interface heights [kall]
 * in HOST memory (the contents of GRD_gz.dat / GRD_gzh.dat read by
 * GRD_Input_vgrid, mod_debug.cpp:189-195).  Allocates all device workspace;
 * no later call allocates.  Uses the current CUDA device.  Returns
 * NSW6_ERR_TOO_LARGE when gall * kall * lall_max >= 2^32. */
int nsw6_create(nsw6_handle** h, int gall, int kall, int lall_max, const double* gz, const double* gzh);
int nsw6_destroy(nsw6_handle* h);

int nsw6_set_params(nsw6_handle* h, const nsw6_params* p);
int nsw6_get_params(const nsw6_handle* h, nsw6_params* p);

/* Scheme switches of NSW6 that the reference selects in mp_nsw6_init
 * (mod_mp_nsw6.cpp:276-434) and in globals (mod_mp_nsw6.cpp:127-132,
 * problemsize.cpp:39).  1 = on; nsw6_default_options gives the reference's
 * configuration {1, 1, 1, 0, 0, 0}. */
typedef struct nsw6_options {
  int roh2014;          /* Roh and Satoh (2014) snow (Roh_flag): its moments and N0g, As, Bs, Esi, Egi,
                           Egs (:345-357); 0 = the classic snow moments (:975-992) and the
                           GlobalParams values (mod_mp_nsw6.h:16-123)                              */
  int explicit_icegen;  /* OPT_EXPLICIT_ICEGEN: Pigen, Pidep, Pihom, Pihtr, Pisub, Pimlt and the
                           liquid saturation adjustment; 0 = Bergeron process (:1239-1247,
                           Bergeron_param :1834-1890) and the mixed-phase adjustment
                           satadjust_all (mod_satadjust.cpp:620-769) between 233.16 K and 273.16 K
                           (:648-661).  roh2014 = 1 forces it on, as mp_nsw6_init does.            */
  int kk2000;           /* qr_aut_acc_type "KK2000"; 0 = Berry (1968) autoconversion and the
                           original accretion (:1091-1099, :1145-1160)                              */
  int qi_sediment;      /* precip_transport_type "4WATER": cloud ice sediments with its fall speed
                           Vti (:1073-1075); 0 = "3WATER"                                          */
  int kin2kin;          /* PRCIP_TRN_ECORRECT "KIN2KIN": the transported kinetic energy rescales the
                           momentum (mod_precip_transport.cpp:1012-1068); 0 = "KIN2EIN"           */
  int aerosol_indirect; /* OPT_INDIR: cloud number max(unccn 1e-6, Nc_def) per cell (:676-679); the
                           unccn argument is then read                                             */
} nsw6_options;

void nsw6_default_options(nsw6_options* o);

/* Selects the scheme switches for the following calls of the handle.  Any
 * non-default switch runs the step (FP64, or mixed precision with
 * mp_driver_mixed / nsw6_set_precision(h, 1)) in the kernels built with the
 * switched branches; with one set, nsw6_set_precision(h, 2),
 * nsw6_set_math(h, 1) and mp_driver_tlm under nsw6_set_adjoint_mode(h, 1)
 * (the serial column step) return NSW6_ERR_UNSUPPORTED. */
int nsw6_set_options(nsw6_handle* h, const nsw6_options* o);
int nsw6_get_options(const nsw6_handle* h, nsw6_options* o);

/* Stream (cudaStream_t, may be 0) on which all work of the handle runs. */
int nsw6_set_stream(nsw6_handle* h, void* stream);

/* When sync_check is non-zero (the default) every mp_driver call waits for
 * its work and returns the device status (like the reference, whose
 * mp_driver ends with Kokkos::fence).  When zero, calls return after
 * enqueueing; read the status with nsw6_last_error. */
int nsw6_set_sync_check(nsw6_handle* h, int sync_check);

/* Newton iteration limit of the saturation adjustment (reference: itelim = 100,
 * mod_satadjust.cpp:809). */
int nsw6_set_itelim(nsw6_handle* h, int itelim);

/* Transcendental functions of the step: 0 (default) table-driven FP64
 * exp/log/pow written for this library (about one unit in the last place),
 * 1 the CUDA math library.  Both agree with the reference to the stated
 * tolerance; mode 1 exists to separate their effects in checks. */
int nsw6_set_math(nsw6_handle* h, int mode);

/* Evaluates the step's table-driven exp (fn 0), log (fn 1) or pow (fn 2,
 * x^y) on n device-resident inputs, for accuracy checks. */
int nsw6_eval_math(nsw6_handle* h, int fn, const double* x, const double* y, double* out, int n);

/* Precision of the step for every entry point of this handle: 0 (default) the
 * plain FP64 step; 1 the mixed-precision step: saturation values, process
 * rates, limiters, tendencies, fall speeds, effective radii and departure
 * distances in FP32, while the negative filter, the tracer and internal-
 * energy budgets, the flux sums of the transport and the saturation-
 * adjustment Newton iteration with its vapour pressure stay FP64; 2 the FP64
 * step evaluated one column per thread by the code the tangent-linear and
 * adjoint kernels are built from (bitwise equal to 0; for checking them;
 * device arrays only: mp_driver_argv with host = 1 returns
 * NSW6_ERR_UNSUPPORTED in this mode).  No counterpart in the reference (FP64
 * only). */
int nsw6_set_precision(nsw6_handle* h, int mode);

/* Per-kernel timing with CUDA events recorded on the handle's stream around
 * each kernel of every step (0 = off, the default). */
int nsw6_set_timing(nsw6_handle* h, int on);

/* Synchronises and returns the kernel time accumulated since the previous
 * read, in milliseconds: t[0] cell kernel, t[1] column kernel (n >= 2), and
 * the number of steps timed.  Resets the accumulators. */
int nsw6_read_timing(nsw6_handle* h, double* t, int n, int* steps);

/* Synchronises the handle's stream and returns the status of the work issued
 * since the previous call; *k, *g, *l and *iters (any may be NULL) give the
 * first failing cell.  Clears the device status word. */
int nsw6_last_error(nsw6_handle* h, int* k, int* g, int* l, int* iters);

const char* nsw6_strerror(int status);

/* Row stride, in doubles, of precip, ISO1_precip and ISO2_precip in the
 * per-region calls mp_driver and mp_driver_mixed: row 1 (snow and graupel)
 * starts `ld` doubles after row 0 (rain).  The reference harness passes
 * subview(precip_mp, ALL, l, 0, ALL) of its [2][lall][1][gall] array
 * (src/main.cpp:37, 220-222), whose rows are lall * gall apart: with
 * ld = lall * gall the per-region call takes that subview's data pointer as it
 * is.  0 (the default) means gall, a contiguous [2][gall] array; 0 < ld < gall
 * is rejected.  The batched, host-memory, multi-step and derivative entry
 * points keep the all-regions layout [2][lall][gall]. */
int nsw6_set_precip_stride(nsw6_handle* h, long long ld);

/* One NSW6 step on one region: replaces MP_DRIVER::mp_driver
 * (src/mod_mp_driver.cpp:335-388), same arguments in the same order.
 * 2-D fields are [kall][gall], tracer fields [6][kall][gall] (QV QC QR QI QS
 * QG), precip/ISO1_precip/ISO2_precip [2][gall] (row 1 gall doubles after row
 * 0, or as set by nsw6_set_precip_stride), precip_rhoe..precip_rhokin and
 * ix..jz [gall], rctop/rwtop/tctop [1][gall].  w, unccn, frhoge_af,
 * frhogqv_af, frhoge_rad, rhogqke, zh, ct and CBMFX are accepted and unused,
 * as in the reference. */
int mp_driver(nsw6_handle* h, int l_region,
              double* rhog, double* rhogvx, double* rhogvy, double* rhogvz, double* rhogw, double* rhoge,
              double* rhogq,
              const double* vx, const double* vy, const double* vz, const double* w, const double* unccn,
              double* rho, double* tem, double* pre,
              double* q, double* qd,
              double* precip, double* ISO1_precip, double* ISO2_precip,
              double* precip_rhoe, double* precip_lh_heat, double* precip_rhophi, double* precip_rhokin,
              double* re_liquid, double* re_solid, double* re_cld,
              double* rctop, double* rwtop, double* tctop,
              const double* frhoge_af, const double* frhogqv_af, const double* frhoge_rad, const double* rhogqke,
              const double* gsgam2, const double* gsgam2h, const double* gam2, const double* gam2h,
              const double* ix, const double* iy, const double* iz,
              const double* jx, const double* jy, const double* jz,
              const double* z, const double* zh,
              double dt, double ct,
              double* GDCLW, double* GDCFRC, double* GPREC, const double* CBMFX);

/* mp_driver in the mixed precision of nsw6_set_precision(h, 1), for this call
 * only; same arguments. */
int mp_driver_mixed(nsw6_handle* h, int l_region,
                    double* rhog, double* rhogvx, double* rhogvy, double* rhogvz, double* rhogw, double* rhoge,
                    double* rhogq,
                    const double* vx, const double* vy, const double* vz, const double* w, const double* unccn,
                    double* rho, double* tem, double* pre,
                    double* q, double* qd,
                    double* precip, double* ISO1_precip, double* ISO2_precip,
                    double* precip_rhoe, double* precip_lh_heat, double* precip_rhophi, double* precip_rhokin,
                    double* re_liquid, double* re_solid, double* re_cld,
                    double* rctop, double* rwtop, double* tctop,
                    const double* frhoge_af, const double* frhogqv_af, const double* frhoge_rad,
                    const double* rhogqke,
                    const double* gsgam2, const double* gsgam2h, const double* gam2, const double* gam2h,
                    const double* ix, const double* iy, const double* iz,
                    const double* jx, const double* jy, const double* jz,
                    const double* z, const double* zh,
                    double dt, double ct,
                    double* GDCLW, double* GDCFRC, double* GPREC, const double* CBMFX);

/* All lall regions in one launch sequence, arrays in the reference harness's
 * all-regions layout (src/main.cpp:19-90): [lall][kall][gall] fields,
 * [lall][6][kall][gall] tracers, [2][lall][gall] precipitation (the
 * precip_mp layout with ADM_KNONE = 1), [lall][gall] column fields and
 * [lall][1][gall] cloud-top fields.  The cross-column reductions of the
 * sedimentation scheme (vadv1d_prep, mod_vadv1d.cpp:316-353) stay per region,
 * so the result equals lall mp_driver calls. */
int mp_driver_batched(nsw6_handle* h, int lall,
                      double* rhog, double* rhogvx, double* rhogvy, double* rhogvz, double* rhogw, double* rhoge,
                      double* rhogq,
                      const double* vx, const double* vy, const double* vz, const double* w, const double* unccn,
                      double* rho, double* tem, double* pre,
                      double* q, double* qd,
                      double* precip, double* ISO1_precip, double* ISO2_precip,
                      double* precip_rhoe, double* precip_lh_heat, double* precip_rhophi, double* precip_rhokin,
                      double* re_liquid, double* re_solid, double* re_cld,
                      double* rctop, double* rwtop, double* tctop,
                      const double* frhoge_af, const double* frhogqv_af, const double* frhoge_rad,
                      const double* rhogqke,
                      const double* gsgam2, const double* gsgam2h, const double* gam2, const double* gam2h,
                      const double* ix, const double* iy, const double* iz,
                      const double* jx, const double* jy, const double* jz,
                      const double* z, const double* zh,
                      double dt, double ct,
                      double* GDCLW, double* GDCFRC, double* GPREC, const double* CBMFX);

/* Same as mp_driver_batched with the 50 array arguments passed as an array
 * of pointers in the reference order (args[0] = rhog ... args[49] = CBMFX).
 * When `host` is non-zero the pointers are HOST memory: the call copies the
 * inputs to device workspace, runs the step and copies the outputs back
 * (synchronous), pipelined by region so copies overlap the kernels.  When all
 * 50 arrays are page-locked (cudaHostAlloc / cudaHostRegister) the pipeline is
 * captured into a CUDA graph on the first call and replayed on later calls
 * (re-captured when the arrays, lall, dt, parameters or settings change);
 * pageable arrays take the direct path.  Both give the device entry's result
 * bit for bit.  This is the entry point a ctypes/cffi/FFI binding uses. */
int mp_driver_argv(nsw6_handle* h, int lall, double* const* args, double dt, double ct, int host);

/* Bytes one mp_driver_argv(host = 1) call on lall regions copies to the
 * device and back with the handle's current settings.  Every argument the
 * step reads is copied in whole except q, of which only QV is read (QC..QG
 * are formed from rhogq), and rhoge, of which only the two halo levels are
 * read (the interior levels' are formed from tem, rhog and q); every argument
 * it writes is copied back whole.  No counterpart in the reference. */
int nsw6_host_copy_bytes(const nsw6_handle* h, int lall, unsigned long long* h2d, unsigned long long* d2h);

/* nsteps consecutive steps of mp_driver_argv (device pointers) on the same
 * arrays, the state evolving in place as in the reference harness's
 * SET_iteration loop (src/main.cpp:261-319).  The step (three memsets and the
 * three kernels) is captured once into a CUDA graph on a stream of the handle
 * and replayed nsteps times on the handle's stream; the graph is kept and
 * re-captured when the arrays, lall, dt, the parameters or the precision /
 * math / itelim settings change.  The status word is checked once, after the
 * last step.  No counterpart in the reference. */
int mp_driver_steps(nsw6_handle* h, int lall, double* const* args, double dt, double ct, int nsteps);

/* ---------------------------------------------------------------------------
 * Tangent-linear and adjoint steps (no counterpart in the reference).
 *
 * Both linearise the FP64 step around the state `args` (the 50 arrays of
 * mp_driver_argv, device pointers, all-regions layout, lall regions).  The
 * derivatives follow the branch each switch and limiter takes; the departure
 * cells and flux-integral bounds of the sedimentation are held fixed; the
 * saturation-adjustment temperature is differentiated implicitly at its
 * converged value.  Parameters are the seven of nsw6_params in their order
 * (beta_saut, qicrt_saut, Cr, Cs, Cg, ice_nuc, kk_aut).  Any kall the handle
 * takes (kall <= 48 with nsw6_set_adjoint_mode 1, whose serial column step
 * holds a column per thread, and takes no scheme switch).  Every scheme
 * switch is taken (kk2000 = 0, aerosol_indirect = 1, roh2014 = 0,
 * explicit_icegen = 0 with the mixed-phase saturation adjustment,
 * differentiated implicitly like the liquid one, qi_sediment with cloud ice
 * as a fourth sedimenting tracer, kin2kin; the adjoint then records the cell
 * physics, and with explicit_icegen = 0 or kin2kin the last column stage, on
 * tapes).
 *
 * mp_driver_tlm: advances `args` by one step (the FP64 step's outputs bit for
 *   bit) and maps the tangents in `targs` (50 device pointers, same layouts;
 *   on entry dx, on exit dy) : dy = (dM/dx) dx + (dM/dp) dp, with dparams[7]
 *   a host array (NULL: no parameter tangent).  Every cell is evaluated in
 *   forward mode (value and tangent) by its own thread, in the same
 *   level-parallel stages as the adjoint; nsw6_set_adjoint_mode 1 selects the
 *   serial column step over the same arithmetic instead (a check).
 *
 * mp_driver_adjoint: `args` is the state BEFORE the step and is not changed.
 *   `aargs` (50 device pointers): on entry the adjoints of the step's outputs,
 *   on exit the adjoints of its inputs -- replaced for the arguments the step
 *   both reads and writes, added to for the arguments it only reads, zero for
 *   the arguments it only writes.  dparams[7] (host, may be NULL): the
 *   parameters' adjoint is added to it.  Every cell is differentiated by its
 *   own thread: the column phase in four level-parallel stages whose input
 *   adjoints are added with atomics (so the last bits depend on their order),
 *   the cell physics per cell, each by a hand-written reverse sweep.  With
 *   nsw6_set_precision(h, 1) (the mixed-precision step) the cell physics is
 *   that step's: FP32 rates and FP32 rate adjoints, FP64 budgets, and the
 *   step's FP32 departure distances; the other column stages and the
 *   accumulation of the state and parameter adjoints stay FP64 (the 12-step
 *   window with a mixed forward uses this); any other
 *   precision, a scheme switch or nsw6_set_adjoint_mode 1 linearise the FP64
 *   step.  The first call allocates the work fields and keeps them in the
 *   handle: about 300 doubles per cell for lall_max regions (nsw6_set_adjoint_mode 1 adds
 *   tapes: about 2.6 GB for the stages and 32 bytes per recorded operation of
 *   the cell physics for 58,368 cells at a time). */
int mp_driver_tlm(nsw6_handle* h, int lall, double* const* args, double* const* targs, const double* dparams,
                  double dt, double ct);

/* Implementation of mp_driver_adjoint and mp_driver_tlm: 0 (default) the
 * hand-written reverse sweeps (no tape), the cell physics' from a checkpoint
 * of its costly forward values (49 doubles per cell, kept in the handle), and
 * the staged tangent-linear step; 1 the operations of the cell physics and of
 * the column stages S1, S2, S4 recorded on per-cell tapes and swept back (the
 * operator-overloading form, for checking the hand-written ones), and the
 * tangent-linear step on the serial column step; 2 as 0, and the hand-written forward
 * the checkpoint comes from is also checked against the step's cell physics
 * on every cell: a cell whose outputs differ in any bit ends the call with
 * NSW6_ERR_CHECK (nsw6_last_error's iters: the first differing output). */
int nsw6_set_adjoint_mode(nsw6_handle* h, int mode);
int mp_driver_adjoint(nsw6_handle* h, int lall, double* const* args, double* const* aargs, double* dparams,
                      double dt, double ct);

/* ---------------------------------------------------------------------------
 * mp_driver_noalloc: one NSW6 step on one region that allocates nothing.
 *
 * No counterpart in the reference (its mp_driver allocates some 45 temporary
 * Views on every call, src/mod_mp_driver.cpp:394-418).  It is for callers that
 * must not call cudaMalloc / cudaFree, or any routine that allocates device
 * memory, inside their time loop: cudaMalloc and cudaFree synchronise the
 * whole device and stall every other stream, and in a process where another
 * allocator (a framework's caching allocator, a fixed memory pool) already
 * holds the device memory a fresh cudaMalloc can fail mid-run.  Such a caller
 * cannot create an nsw6_handle, which allocates its workspace.
 *
 * The workspace is a fixed file-scope device array inside the library (about
 * 110 MB, present on every device the library is loaded on).  Limits: kall in
 * [5, 160] and gall * kall <= NSW6_NOALLOC_MAX_CELLS; larger regions return
 * NSW6_ERR_TOO_LARGE before anything is issued.
 *
 * gz, gzh: HOST arrays of kall heights (the contents of GRD_gz.dat /
 * GRD_gzh.dat).  params: NULL for the defaults.  args: the 50 arrays of one
 * region in the reference order (args[0] = rhog ... args[49] = CBMFX), CUDA
 * device pointers, per-region layout as for mp_driver.  stream: a
 * cudaStream_t (NULL = the default stream).  The call issues its work on
 * `stream`, then synchronises it and returns the step's status
 * (NSW6_ERR_NOCONV / NSW6_ERR_NAN as mp_driver).
 *
 * Set-up: every call looks up the scratch array's device address on the
 * current device (cudaGetSymbolAddress; the first call on a device may load
 * the library's device code there).  The call ends by reading the step's
 * status back and synchronising `stream`, so it cannot run on a stream that
 * is being captured into a CUDA graph: it then returns NSW6_ERR_UNSUPPORTED
 * before issuing anything.
 *
 * Zero state: nothing has to be zero before a call.  Each call writes the grid
 * metrics and fast-math tables into the scratch, resets the status word to 0
 * and the departure-distance extrema keys to 0 / all ones, and every
 * departure distance the step reads is written by the same call first.
 *
 * Concurrency: all calls in the process share one scratch array per device.
 * Calls that overlap in time (from several host threads, or on several streams
 * of one device without ordering between them) race on it and give wrong
 * results; serialise them. */
#define NSW6_NOALLOC_MAX_CELLS 2097152
int mp_driver_noalloc(int gall, int kall, const double* gz, const double* gzh, const nsw6_params* params,
                      double* const* args, double dt, double ct, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NSW6_H */
