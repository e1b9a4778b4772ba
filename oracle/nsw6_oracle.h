/* CPU restatement of one NICAM NSW6 microphysics step (TEST INFRASTRUCTURE ONLY).
 *
 * This is the oracle the CUDA implementation is checked against.  It restates,
 * pass by pass, the reference's Kokkos code path of MP_DRIVER::mp_driver
 * (src/mod_mp_driver.cpp:335-613) with MP_TYPE = "NSW6" and the configuration
 * hard-wired by mp_nsw6_init (src/mod_mp_nsw6.cpp:276-434).  It is pinned
 * against the reference's own sources compiled with a host Kokkos shim
 * (oracle/build_ref.py), with which it agrees bit for bit on this host.
 *
 * The shipped library never links this code; only tests, the golden-fixture
 * script and the CPU-baseline leg of bench.py do.
 */
#ifndef NSW6_ORACLE_H
#define NSW6_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Tunable NSW6 parameters, same order and meaning as nsw6_params in
 * include/nsw6.h. */
typedef struct nsw6o_params {
  double beta_saut;   /* ice->snow autoconversion rate        (mod_mp_nsw6.cpp:287-294) */
  double qicrt_saut;  /* ice->snow autoconversion threshold   (mod_mp_nsw6.h:87)        */
  double Cr;          /* rain fall-speed coefficient          (mod_mp_nsw6.h:27)        */
  double Cs;          /* snow fall-speed coefficient          (mod_mp_nsw6.h:28)        */
  double Cg;          /* graupel fall-speed coefficient       (mod_mp_nsw6.cpp:337)     */
  double ice_nuc;     /* ice nucleation coefficient in Qi0    (mod_mp_nsw6.cpp:1083)    */
  double kk_aut;      /* KK2000 autoconversion rate           (mod_mp_nsw6.cpp:1154)    */
} nsw6o_params;

/* Defaults of the active configuration. */
void nsw6o_default_params(nsw6o_params* p);

/* One mp_driver call on one region.  `a` holds the 50 array arguments of the
 * reference mp_driver in its order (mod_mp_driver.h:71-124), contiguous:
 * [kall][gall] fields, [6][kall][gall] tracers, [2][gall] precipitation,
 * [gall] or [1][gall] column fields.  gz/gzh are the full-level and interface
 * heights [kall].  Returns 0, or 2 when the saturation-adjustment Newton
 * iteration did not converge (status[1..3] = k, g, iterations of the first
 * such cell), or 1 on bad arguments. */
int nsw6o_mp_driver(int gall, int kall, const double* gz, const double* gzh,
                    const nsw6o_params* p, double* const* a, double dt, double ct,
                    int itelim, int* status);

/* Threads used by the OpenMP build (1 for the serial build). */
int nsw6o_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
