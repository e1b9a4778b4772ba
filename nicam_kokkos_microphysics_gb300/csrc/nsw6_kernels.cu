// GB300 (sm_103a) kernels of one NSW6 microphysics step, FP64.
//
// Three kernels per step (plus three memsets: the extrema buffers and the
// saturated-cell list's count):
//
//  nsw6_cell_kernel    one CTA = CELL_TG columns x all interior levels of one
//                      region.  Per cell: negative filter, saturation values,
//                      Bergeron parameters, the NSW6 process rates, the
//                      RHOGQ/RHOGE/TEM updates and the fall speeds.  Then, per
//                      column, the sedimentation departure distances of
//                      vadv1d_prep for QR/QS/QG on full and half levels and
//                      their per-level extrema, reduced over the region with
//                      exact order-preserving 64-bit atomics.
//
//  nsw6_column_kernel  one CTA = COL_TG columns x all levels, column state in
//                      shared memory.  Departure cells, the 24 flux integrals of
//                      vadv1d_getflux_new, the transport tendencies, surface
//                      precipitation, the KIN2EIN energy correction, the final
//                      thermodynamic state and the closing negative filter; the
//                      cells the saturation adjustment finds saturated are
//                      listed instead.
//
//  nsw6_satadj_kernel  one thread per listed cell: its Newton iteration on T
//                      (the saturation adjustment) and its final state.
//
// The only coupling between columns, the per-level max/min of the departure
// distance over a region (mod_vadv1d.cpp:316-353), is what separates the two
// kernels.
#include <cfloat>
#include <cuda_runtime.h>

#include "nsw6_cell.cuh"
#include "nsw6_common.cuh"
#include "nsw6_fastmath.cuh"

namespace nsw6 {

constexpr int ERR_NOCONV = 3;
constexpr int ERR_NAN = 4;

__device__ __forceinline__ void record_error(DevStatus* st, int code, int k, int g, int l, int iters) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->k = k;
    st->g = g;
    st->l = l;
    st->iters = iters;
  }
}

// ------------------------------------------------------------------ kernel 1
template <class M>
__device__ __forceinline__ M make_math(const double* tab);
template <>
__device__ __forceinline__ FastMath make_math<FastMath>(const double* tab) {
  return FastMath{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
}
template <>
__device__ __forceinline__ LibMath make_math<LibMath>(const double*) {
  return LibMath{};
}
template <>
__device__ __forceinline__ FloatMath make_math<FloatMath>(const double*) {
  return FloatMath{};
}

// Shared memory of the cell kernel: fall speeds [ntr][K][CELL_TG] (type R; 3
// sedimenting tracers, 4 in the kernel with the scheme switches), the grid
// block [GF_COUNT][K] and the fast-math tables (doubles), and for R = float
// FP32 copies of the four reciprocal rows the departure distances use.
template <class R>
__host__ __device__ constexpr size_t cell_vts_doubles(int K, int nv = 3) {
  return (nv * (size_t)K * CELL_TG * sizeof(R) + sizeof(double) - 1) / sizeof(double);
}

// OPT: the kernel with the scheme switches (FP64 only): the switched branches
// of nsw6_cell, the CCN input, and the ice fall speed with its departure
// distances when QI sediments.
template <class M, class R, bool OPT = false>
__global__ void __launch_bounds__(CELL_THREADS, 2) nsw6_cell_kernel(Problem P, ConstsT<R> C) {
  constexpr bool kMixed = sizeof(R) == sizeof(float);
  constexpr int NV = OPT ? 4 : 3;            // fall-speed rows in shared memory
  const int ntr = OPT ? P.ntr : 3;          // sedimenting tracers of this call
  extern __shared__ double sm[];
  const int G = P.gall, K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const int l = blockIdx.y;
  const int g0 = blockIdx.x * CELL_TG;
  const size_t KG = (size_t)K * G;
  const size_t off = (size_t)l * KG;
  const size_t offq = (size_t)l * NQ * KG;
  R* vts = reinterpret_cast<R*>(sm);                   // [ntr][K][CELL_TG] fall speeds, tracer order
  // grid metrics and FastMath tables: staged in shared memory, or, in the
  // kernel with the scheme switches for columns deeper than CELL_SMEM_KMAX,
  // read from global memory (through L1)
  const bool stage = !OPT || K <= CELL_SMEM_KMAX;
  double* sgrid = sm + cell_vts_doubles<R>(K, NV);     // [GF_COUNT][K]
  double* stab = sgrid + (stage ? GF_COUNT * K : 0);   // [FM_TABLE_DOUBLES]
  const double* grid = stage ? sgrid : P.grid;
  const double* tab = stage ? stab : P.fmtab;
  float* gridf = reinterpret_cast<float*>(stab + (stage ? FM_TABLE_DOUBLES : 0));  // [4][K], mixed only
  unsigned short* perm = reinterpret_cast<unsigned short*>(gridf + 4 * K);  // [nlev * CELL_TG], FP64 only
  unsigned char* key = reinterpret_cast<unsigned char*>(perm + (K - 2) * CELL_TG);
  R* whs = reinterpret_cast<R*>(                                          // [K][CELL_TG] half-level velocities
      (reinterpret_cast<uintptr_t>(key + (K - 2) * CELL_TG) + 15) & ~(uintptr_t)15);
  __shared__ int bucket[33];

  for (int c = threadIdx.x; c < NV * K * CELL_TG; c += blockDim.x) vts[c] = R(0.0);
  if (stage) {
    for (int c = threadIdx.x; c < GF_COUNT * K; c += blockDim.x) sgrid[c] = P.grid[c];
    if (!kMixed)
      for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) stab[c] = P.fmtab[c];
  }
  if (kMixed) {
    const int rows[4] = {GF_RDGZ, GF_RDGZH, GF_RDZS, GF_RDZSH};
    for (int c = threadIdx.x; c < 4 * K; c += blockDim.x) gridf[c] = (float)P.grid[rows[c / K] * K + c % K];
  }
  __syncthreads();
  const M mth = make_math<M>(tab);

  const int nlev = kmax - kmin + 1;
  const int ncell = nlev * CELL_TG;
  // FP64: the tile's cells are grouped by the hydrometeors they hold (snow,
  // rain, graupel, ice, cloud water: the blocks nsw6_cell skips when a species
  // is absent), so that warps are uniform and skip those blocks together.  The
  // order only decides which thread computes which cell.
  int nvalid = ncell;
  if (!kMixed) {
    for (int c = threadIdx.x; c < 33; c += blockDim.x) bucket[c] = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
      const int k = kmin + c / CELL_TG;
      const int g = g0 + c % CELL_TG;
      int kk = 32;   // columns past the region's end go last
      if (g < G) {
        const size_t iq = offq + (size_t)k * G + g;
        kk = (gt_z(P.rhogq[iq + (size_t)I_QS * KG]) ? 16 : 0) | (gt_z(P.rhogq[iq + (size_t)I_QR * KG]) ? 8 : 0) |
             (gt_z(P.rhogq[iq + (size_t)I_QG * KG]) ? 4 : 0) | (gt_z(P.rhogq[iq + (size_t)I_QI * KG]) ? 2 : 0) |
             (gt_z(P.rhogq[iq + (size_t)I_QC * KG]) ? 1 : 0);
      }
      key[c] = (unsigned char)kk;
      atomicAdd(&bucket[kk], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int run = 0;
      for (int b = 0; b < 33; ++b) {
        const int n = bucket[b];
        bucket[b] = run;
        run += n;
      }
    }
    __syncthreads();
    nvalid = bucket[32];   // cells of columns inside the region
    __syncthreads();
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) perm[atomicAdd(&bucket[key[c]], 1)] = (unsigned short)c;
    __syncthreads();
  }
  for (int j = threadIdx.x; j < nvalid; j += blockDim.x) {
    const int c = kMixed ? j : perm[j];
    const int k = kmin + c / CELL_TG;
    const int gx = c % CELL_TG;
    const int g = g0 + gx;
    if (g >= G) continue;
    const size_t i = off + (size_t)k * G + g;
    const size_t iq = offq + (size_t)k * G + g;
    CellIn in;
    in.rhog = P.rhog[i];
    in.tem = P.tem[i];
    in.gsgam2 = P.gsgam2[i];
    in.q0 = P.q[iq];
#pragma unroll
    for (int n = 0; n < 6; ++n) in.rhogq[n] = P.rhogq[iq + (size_t)n * KG];
    in.unccn = (OPT && P.unccn) ? P.unccn[i] : 0.0;   // required only with the aerosol switch
    CellOut o;
    nsw6_cell<M, R, double, OPT>(C, mth, P.dt, P.rdt, in, o);
    P.rhog[i] = o.rhog;
    P.rhoge[i] = o.rhoge;
    P.tem[i] = o.tem;
#pragma unroll
    for (int n = 0; n < 6; ++n) P.rhogq[iq + (size_t)n * KG] = o.rhogq[n];
#pragma unroll
    for (int n = 1; n < 6; ++n) P.q[iq + (size_t)n * KG] = o.q[n];
    P.re_liquid[i] = o.rceff;
    P.re_cld[i] = o.rceff_cld;
    // tracer order of the transport: QR, (QI,) QS, QG
    vts[(0 * K + k) * CELL_TG + gx] = R(o.Vtr);
    if (ntr == 4) vts[(1 * K + k) * CELL_TG + gx] = R(o.Vti);
    vts[((ntr - 2) * K + k) * CELL_TG + gx] = R(o.Vts);
    vts[((ntr - 1) * K + k) * CELL_TG + gx] = R(o.Vtg);
    if (k == kmax) {
      // The reference writes the cloud-top scalars from every level in parallel
      // (mod_mp_nsw6.cpp:1579-1592); the sequential order, in which the top
      // interior level is written last, is used.  TagUpdateCLD, :710-726.
      const size_t ic = (size_t)l * G + g;
      P.rctop[ic] = o.rctop;
      P.tctop[ic] = o.tctop;
      const double sw = (0.5 + copysign(0.5, o.tctop - TEM00));
      P.rwtop[ic] = (sw)*o.rctop + (1.0 - sw) * UNDEF;
    }
  }
  __syncthreads();

  // Departure distances (vadv1d_prep) and their per-level region extrema.
  // Row s = t + ntr*half: t = the sedimenting tracer; half = 0 full levels
  // (mkmin = kmin, dz = dgz), 1 half levels (mkmin = kmin+1, dz = dgzh,
  // wp = Vtermh).
  const R* rdgz;
  const R* rdgzh;
  const R* rdzs;
  const R* rdzsh;
  if constexpr (kMixed) {
    rdgz = gridf;
    rdgzh = gridf + K;
    rdzs = gridf + 2 * K;
    rdzsh = gridf + 3 * K;
  } else {
    rdgz = grid + GF_RDGZ * K;
    rdgzh = grid + GF_RDGZH * K;
    rdzs = grid + GF_RDZS * K;
    rdzsh = grid + GF_RDZSH * K;
  }
  const R dtR = R(P.dt), hdt2R = R(P.hdt2), sdt3R = R(P.sdt3);
  // one row at a time: its half-level velocities wh(j) first (each is used by
  // three departure distances), then the distances
  const int nrow = 2 * ntr;
  for (int s = 0; s < nrow; ++s) {
    const int t = s % ntr;
    const int half = s / ntr;
    const int mkmin = half ? kmin + 1 : kmin;
    for (int c = threadIdx.x; c < K * CELL_TG; c += blockDim.x) {
      const int j = c / CELL_TG, gx = c % CELL_TG;
      if (j < mkmin - 1 || j > kmax + 1) continue;
      const R* col = vts + t * K * CELL_TG + gx;
      R v;
      if (!half) {
        auto wp = [&](int jj) { return col[jj * CELL_TG]; };
        v = vadv_wh<R>(wp, j, mkmin, kmax);
      } else {
        // Vtermh, mod_precip_transport.cpp:847-861
        auto wp = [&](int jj) {
          return (jj >= kmin + 1 && jj <= kmax - 1) ? R(0.5) * (col[jj * CELL_TG] + col[(jj - 1) * CELL_TG]) : R(0.0);
        };
        v = vadv_wh<R>(wp, j, mkmin, kmax);
      }
      whs[c] = v;
    }
    __syncthreads();
  for (int c = threadIdx.x; c < K * CELL_TG; c += blockDim.x) {
    const int k = c / CELL_TG;
    const int gx = c % CELL_TG;
    if (k < mkmin || k > kmax) continue;  // uniform across the warp (CELL_TG == 32)
    const int g = g0 + gx;
    const bool valid = g < G;
    double z = 0.0;
    if (valid) {
      auto wh = [&](int j) { return whs[j * CELL_TG + gx]; };
      z = half ? double(vadv_zdis_wh<R>(wh, rdgzh, rdzsh, k, mkmin, dtR, hdt2R, sdt3R))
               : double(vadv_zdis_wh<R>(wh, rdgz, rdzs, k, mkmin, dtR, hdt2R, sdt3R));
      P.zdis[((size_t)l * nrow + s) * KG + (size_t)k * G + g] = z;
    }
    // NaN never wins the reference's comparisons, so it is left out
    const bool use = valid && !is_nan_bits(z);
    unsigned long long kmx = use ? order_key(z) : 0ull;
    unsigned long long kmn = use ? order_key(z) : ~0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long a = __shfl_xor_sync(0xffffffffu, kmx, o);
      const unsigned long long b = __shfl_xor_sync(0xffffffffu, kmn, o);
      kmx = a > kmx ? a : kmx;
      kmn = b < kmn ? b : kmn;
    }
    if ((threadIdx.x & 31) == 0) {
      const size_t e = ((size_t)l * nrow + s) * K + k;
      if (kmx != 0ull) atomicMax(&P.zmax[e], kmx);
      if (kmn != ~0ull) atomicMin(&P.zmin[e], kmn);
    }
  }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ kernel 2
// Shared-memory field slots, each [K][COL_TG] doubles.
// S_DQI (the tendency of sedimenting QI) exists in the kernel with the scheme
// switches only.
// Above this many levels the column kernel with the scheme switches reads the
// FastMath tables (8 KB) from global memory (they stay in L1) instead of
// staging them in shared memory, so that its tile fits at MAX_KALL levels.
constexpr int COL_FMTAB_SMEM_KMAX = 128;

enum ColSlot {
  S_KINH, S_KINV, S_DRHOE, S_DRHOPHI, S_DKINH, S_DKINV, S_DRHOGU, S_DRHOGV, S_DRHOGW,
  S_DQR, S_DQS, S_DQG, S_RHOF, S_F, S_RGS, S_BASE, S_VI, S_VJ, S_COUNT,
  S_DQI = S_COUNT, S_COUNT_OPT
};

struct ColumnShared {
  double* f;         // [S_COUNT (S_COUNT_OPT)][K][COL_TG]
  double* grid;      // [GF_COUNT][K]
  double* colacc;    // [6][COL_TG]: precip0, precip1, lh_heat, rhoe, rhophi, rhokin
  int* bmin;         // [2 ntr][K] (room for 8 rows with the switches)
  int* bmax;         // [2 ntr][K]
  unsigned char* kc; // [K][COL_TG]
};

// Departure cell of vadv1d_prep for one cell (mod_vadv1d.cpp:355-389).  The
// reference's tmp = k2 * copysign(1, dep - zh(k2)) * copysign(1, zh(k2+1) - dep)
// is k2 when both signs agree and -k2 otherwise; the sign of a difference of
// two doubles is their comparison, so the test is exact integer logic.
//
// The comparisons run on the integer pipe: zk holds cmp_key of the interface
// heights zh, and for non-NaN doubles a >= b exactly when their keys compare
// so; a NaN departure point makes every comparison false, as in the reference.
__device__ __forceinline__ int departure_cell(const double* zh, const long long* zk, int k, double zdis, int bmn,
                                              int bmx, int mkmin, int mkmax) {
  int kc;
  if (bmn == k && bmx == k) {
    kc = k;
  } else {
    kc = 0;
    const double dep = zh[k] - zdis;
    const long long dk = cmp_key(dep);
    const bool nan = is_nan_bits(dep);
    for (int k2 = bmn; k2 <= bmx; ++k2) {
      const bool s1 = !nan && dk >= zk[k2];
      const bool s2 = !nan && zk[k2 + 1] >= dk;
      const int tmp = (s1 == s2) ? k2 : -k2;
      kc = kc > tmp ? kc : tmp;
    }
  }
  if (kc == 0) kc = mkmin;
  if (kc == mkmax + 1) kc = mkmax;
  return kc;
}

// Flux integral of vadv1d_getflux_new for one cell (mod_vadv1d.cpp:410-449),
// including its small-value filter |f| < EPS -> 0.  In the reference's Kokkos
// lambda the level index is a size_t, so its (k-1)-k2 and k2-k factors are
// evaluated unsigned and never negative; the weight of layer k2 is then
// fact = dz(k2) * 0.25 * ((sign(k2-kc-1)+1) * 2 - 2 * (sign(kc-1-k2)+1)),
// i.e. +dz(k2) above the departure cell, -dz(k2) below it and 0 at it, and
// zdis = zdis0 - fact of the last layer k2 = bmx.
template <int TG>
__device__ __forceinline__ double flux_integral(const double* rhof_col, const double* dz, int k, int kc,
                                                double zdis0, int bmn, int bmx) {
  double f = 0.0, zdis = zdis0;
  if (!(bmn == k && bmx == k)) {
    // the departure cell's own weight is 0 (the reference multiplies by it):
    // adding rhof(kc) * 0 leaves f unchanged and keeps every lane busy
    for (int k2 = bmn; k2 <= bmx; ++k2)
      f = __fma_rn(rhof_col[k2 * TG], k2 > kc ? dz[k2] : (k2 < kc ? -dz[k2] : 0.0), f);
    if (bmx != kc) zdis = zdis0 - (bmx > kc ? dz[bmx] : -dz[bmx]);
  }
  f = __fma_rn(rhof_col[kc * TG], zdis, f);
  // |f| >= EPS on the integer pipe (NaN fails, as the comparison does)
  const long long ab = __double_as_longlong(f) & 0x7fffffffffffffffLL;
  return (ab >= EPS_BITS && ab <= 0x7ff0000000000000LL) ? f : 0.0;
}

// Kinetic energies of the mixed step (FP32): horizontal, 0.5 |rhog v|^2 / rhog
// of a cell, and vertical, 0.5 rhogw^2 / (c2w0 rhog(k) + c2w1 rhog(k-1)) of a
// half level (mod_precip_transport.cpp:744-766, 991-1011).  The same functions
// form the energies before and after the transport, so a column the transport
// leaves unchanged gets a zero KIN2EIN correction, as in the FP64 step.
__device__ __forceinline__ float kin_h_f(float rvx, float rvy, float rvz, float rhog) {
  return __fdiv_rn(0.5f * __fmaf_rn(rvx, rvx, __fmaf_rn(rvy, rvy, __fmul_rn(rvz, rvz))), rhog);
}
__device__ __forceinline__ float kin_v_f(float rw, float c2w0, float c2w1, float rhog, float rhog_below) {
  return __fdiv_rn(0.5f * __fmul_rn(rw, rw), __fmaf_rn(c2w0, rhog, __fmul_rn(c2w1, rhog_below)));
}

// FP32 flux integral of the mixed path (momentum fluxes), same form.
template <int TG>
__device__ __forceinline__ float flux_integral_f(const float* rhof_col, const float* dz, int k, int kc, float zdis0,
                                                 int bmn, int bmx) {
  float f = 0.0f, zdis = zdis0;
  if (!(bmn == k && bmx == k)) {
    for (int k2 = bmn; k2 <= bmx; ++k2)
      f = __fmaf_rn(rhof_col[k2 * TG], k2 > kc ? dz[k2] : (k2 < kc ? -dz[k2] : 0.0f), f);
    if (bmx != kc) zdis = zdis0 - (bmx > kc ? dz[bmx] : -dz[bmx]);
  }
  f = __fmaf_rn(rhof_col[kc * TG], zdis, f);
  return fabsf(f) >= (float)EPS ? f : 0.0f;
}

// Newton iteration of the saturation adjustment of one saturated cell:
// satadjust_liq (mod_satadjust.cpp:771-896, the iteration :840-880) or, with
// the switch, satadjust_all (:620-769, the iteration :686-754).  q holds the
// cell's specific humidities with q[QV] = qsum and q[QC] (and q[QI] with
// satadjust_all) = 0; the iteration leaves the adjusted ones there and
// returns the temperature.  Its range, convergence and finiteness tests run
// on the integer pipe (nsw6_fpcmp.cuh).
template <class M>
__device__ __forceinline__ double satadjust_newton(const Problem& P, const Consts& C, const M& mth, bool ice_adj,
                                                   double tem, double ein_moist, double qsum, double rho_l,
                                                   double qd_l, double* q, int k, int g, int l) {
  bool converged = false;
  int ite;
  if (ice_adj) {
    // satadjust_all, mod_satadjust.cpp:686-754 (CPovR = CVovR = 0, all CVW = CVdry)
    const double UL = C.sat_ulimit, LL = C.sat_llimit;
    for (ite = 0; ite < P.itelim; ++ite) {
      const double alpha = dmin(dmax((tem - LL) / (UL - LL), 0.0), 1.0);
      const double rtem = 1.0 / fp_max_pos(tem, TEM_MIN);
      const double psatl = PSAT0 * mth.exp(C.LovR_liq * (C.RTEM00 - rtem));
      const double psati = PSAT0 * mth.exp(C.LovR_ice * (C.RTEM00 - rtem));
      const double psat = psatl * alpha + psati * (1.0 - alpha);
      const double qsatl = psatl / (rho_l * RVAP * tem);
      const double qsati = psati / (rho_l * RVAP * tem);
      const double qsat = psat / (rho_l * RVAP * tem);
      q[I_QV] = qsat;
      q[I_QC] = (qsum - qsat) * alpha;
      q[I_QI] = (qsum - qsat) * (1.0 - alpha);
      double cv = qd_l * CVDRY;
#pragma unroll
      for (int n = 1; n <= 5; ++n) cv = cv + q[n] * CVDRY;
      const double emoist_new = tem * cv + q[I_QV] * LHV0 - q[I_QI] * LHF0;
      const double dalpha_dT = (!(UL - tem < 0.0) && !(tem - LL < 0.0)) ? 1.0 / (UL - LL) : 0.0;
      const double t2 = tem * tem;
      const double dqsatl_dT = (C.LovR_liq / t2) * qsatl;
      const double dqsati_dT = (C.LovR_ice / t2) * qsati;
      const double dqsat_dT = qsatl * dalpha_dT + dqsatl_dT * alpha - qsati * dalpha_dT + dqsati_dT * (1.0 - alpha);
      const double dqc_dT = (qsum - qsat) * dalpha_dT - dqsat_dT * alpha;
      const double dqi_dT = -(qsum - qsat) * dalpha_dT - dqsat_dT * (1.0 - alpha);
      const double dcv_dT = dqsat_dT * CVDRY + dqc_dT * CVDRY + dqi_dT * CVDRY;
      const double demoist_dT = tem * dcv_dT + cv + dqsat_dT * LHV0 - dqi_dT * LHF0;
      const double dtemp = (emoist_new - ein_moist) / demoist_dT;
      tem = tem - dtemp;
      if (fp_abs_lt(dtemp, C.dtemp_criteria)) {
        converged = true;
        break;
      }
      if (fp_not_finite(tem)) break;
    }
  } else {
    for (ite = 0; ite < P.itelim; ++ite) {
      const double rtem = 1.0 / fp_max_pos(tem, TEM_MIN);
      const double psat = PSAT0 * mth.exp(C.LovR_liq * (C.RTEM00 - rtem));
      const double qsat = psat / (rho_l * RVAP * tem);
      q[I_QV] = qsat;
      q[I_QC] = qsum - qsat;
      double cv = qd_l * CVDRY;
#pragma unroll
      for (int n = 1; n <= 5; ++n) cv = cv + q[n] * CVDRY;
      const double emoist_new = tem * cv + q[I_QV] * LHV0;
      // dqsat/dT = (LovR/T^2 + CVovR/T) qsat with CVovR = 0, and
      // dCVtot/dT = dqsat/dT (CVW(QV) - CVW(QC)) = 0 (all CVW = CVdry)
      const double dqsat_dT = C.LovR_liq * rtem * rtem * qsat;
      const double demoist_dT = cv + dqsat_dT * LHV0;
      const double dtemp = (emoist_new - ein_moist) / demoist_dT;
      tem = tem - dtemp;
      if (fp_abs_lt(dtemp, C.dtemp_criteria)) {
        converged = true;
        break;
      }
      if (fp_not_finite(tem)) break;
    }
  }
  if (!converged) record_error(P.status, fp_not_finite(tem) ? ERR_NAN : ERR_NOCONV, k, g, l, ite);
  return tem;
}

// The final state of one cell after the transport and KIN2EIN: thermodynamics,
// saturation adjustment, negative filter and outputs (mod_mp_driver.cpp:
// 555-612 with mod_thrmdyn.cpp, mod_satadjust.cpp:274-362 and
// mod_mp_nsw6.cpp:1770-1831).  rhog, its reciprocal and rhoge (after KIN2EIN)
// are the cell's; the rest comes from the state arrays.  With newton = false
// (the column kernel) a saturated interior cell is left as it is and true is
// returned, for nsw6_satadj_kernel; every other cell is finished.  With
// newton = true (that kernel) the cell is saturated: the same values are
// formed, the Newton iteration runs and the cell is finished.
template <class M, bool MIX, bool OPT>
__device__ __forceinline__ bool final_cell(const Problem& P, const Consts& C, const M& mth, bool ice_adj, float lovr_f,
                                           size_t i, size_t iq, size_t KG, bool interior, double rhog, double rrhog,
                                           double rhoge, bool newton, int k, int g, int l) {
  double rq[6], q[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] = P.rhogq[iq + (size_t)n * KG];
  // These quotients must be correctly rounded: the saturation adjustment
  // forms qc = qsum - qsat from them, a difference of nearly equal numbers
  // in which one unit in the last place of qsum is already a relative error
  // of 1e-11 when qc is small.
#pragma unroll
  for (int n = 0; n < 6; ++n) q[n] = MIX ? rq[n] * rrhog : div_rn(rq[n], rhog, rrhog);
  const double gsg = P.gsgam2[i];
  double rho = rhog / gsg;
  const double ein = MIX ? rhoge * rrhog : div_rn(rhoge, rhog, rrhog);
  double qd = 1.0;
#pragma unroll
  for (int n = 1; n <= 5; ++n) qd = qd - q[n];
  // THRMDYN_tempre, mod_thrmdyn.cpp:137-180.  Its temperature is replaced
  // by the saturation adjustment's everywhere and its pressure by the
  // negative filter's at interior levels: only the halo levels output it.
  double pre = 0.0;
  if (!interior) {
    double cvt = 0.0, qdl = 1.0;
#pragma unroll
    for (int n = 1; n <= 5; ++n) {
      cvt = cvt + q[n] * CVDRY;
      qdl = qdl - q[n];
    }
    cvt = cvt + qdl * CVDRY;
    const double tem0 = ein / cvt;
    pre = rho * tem0 * (qdl * RDRY + q[I_QV] * RVAP);
  }

  // SATURATION_adjustment (mod_satadjust.cpp:274-362): ice_adjust = false,
  // or true with the switch (cloud ice joins the adjustment)
  double ein_moist, qsum;
  if (ice_adj) {
    ein_moist = ein + q[I_QV] * LHV0 - q[I_QI] * LHF0;
    qsum = q[I_QV] + q[I_QC] + q[I_QI];
    q[I_QI] = 0.0;
  } else {
    ein_moist = ein + q[I_QV] * LHV0;
    qsum = q[I_QV] + q[I_QC];
  }
  q[I_QV] = qsum;
  q[I_QC] = 0.0;
  // q[QC] (and q[QI] in satadjust_all) is +0 now: its terms leave the sums
  // below as they are (no partial sum is -0), so they are not formed
  // MIX: every CVW is CVdry, so the sum is formed first and scaled once
  double cvtot = MIX ? qd : qd * CVDRY;
#pragma unroll
  for (int n = 2; n <= 5; ++n)
    if (n != I_QI || !ice_adj) cvtot = MIX ? cvtot + q[n] : cvtot + q[n] * CVDRY;
  if (MIX) cvtot = cvtot * CVDRY;
  const double rho_l = rho;
  double tem = (ein_moist - q[I_QV] * LHV0) / cvtot;
  if (interior) {
    // satadjust_liq (mod_satadjust.cpp:771-896) or satadjust_all
    // (:620-769)
    double qd_l = 1.0;
#pragma unroll
    for (int n = 2; n <= 5; ++n)
      if (n != I_QI || !ice_adj) qd_l = qd_l - q[n];
    if (newton) {
      tem = satadjust_newton(P, C, mth, ice_adj, tem, ein_moist, qsum, rho_l, qd_l, q, k, g, l);
    } else {
    // is the cell saturated?
    // The test qsum - qsat(tem) > EPS is first decided in FP32 (liquid
    // saturation only, sat_screen_liq); the FP64 test decides the rest.
    int sat = ice_adj ? -1 : sat_screen_liq(tem, rho_l, qsum, lovr_f);
    if (sat < 0) {
      const double rtem = 1.0 / fp_max_pos(tem, TEM_MIN);
      double psat = PSAT0 * mth.exp(C.LovR_liq * (C.RTEM00 - rtem));
      if (ice_adj) {
        const double alpha =
            dmin(dmax((tem - C.sat_llimit) / (C.sat_ulimit - C.sat_llimit), 0.0), 1.0);
        const double psati = PSAT0 * mth.exp(C.LovR_ice * (C.RTEM00 - rtem));
        psat = psat * alpha + psati * (1.0 - alpha);
      }
      const double qsat = psat / (rho_l * RVAP * tem);
      sat = (qsum - qsat > EPS) ? 1 : 0;
    }
    if (sat) return true;
    }
  }
  rq[I_QV] = rhog * q[I_QV];
  rq[I_QC] = rhog * q[I_QC];
  if (ice_adj) rq[I_QI] = rhog * q[I_QI];
  if (!interior) {   // interior levels: rhoge comes from the negative filter below
    cvtot = qd * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cvtot = cvtot + q[n] * CVDRY;
    rhoge = rhog * tem * cvtot;
  }

  // negative_filter (mod_mp_nsw6.cpp:1770-1831), interior levels
  double rhog_o = rhog;
  if (interior) {
    double diffq = 0.0;
    unsigned clamped = 0;   // bit n: rq[n] was negative and is now zero
#pragma unroll
    for (int n = 2; n <= 5; ++n) {
      diffq += rq[n];
      if (lt_z(rq[n])) clamped |= 1u << n;
      rq[n] = maxz(rq[n]);
    }
#pragma unroll
    for (int n = 2; n <= 5; ++n) diffq -= rq[n];
    rq[I_QV] += diffq;
    diffq = rq[I_QV];
    rq[I_QV] = maxz(rq[I_QV]);
    diffq -= rq[I_QV];
    double qdf, cva;
    if (fp_is_zero(diffq) && fp_pos_normal(rhog)) {
      // Nothing removed: rhog (1 - diffq) is rhog exactly, and so are
      // rho = rhog / gsg and the reciprocal formed above.  The quotients of
      // the tracers the filter left as they were are those formed above
      // (QR, QS, QG; QI unless the adjustment set it), and an unsaturated
      // cell's cloud water is +0 = (rhog 0) / rhog.
      const unsigned same = (0x34u | (ice_adj && newton ? 0u : 0x08u) | (newton ? 0u : 0x02u)) & ~clamped;
#pragma unroll
      for (int n = 1; n <= 5; ++n)
        if (!((same >> n) & 1u)) q[n] = MIX ? rq[n] * rrhog : div_rn(rq[n], rhog, rrhog);
      // an unsaturated cell's q[QC] (and q[QI] in satadjust_all) is still +0
      const unsigned zero = newton ? 0u : (ice_adj ? 0x0Au : 0x02u);
      qdf = 1.0;
#pragma unroll
      for (int n = 1; n <= 5; ++n)
        if (!((zero >> n) & 1u)) qdf = qdf - q[n];
      cva = CVDRY;   // MIX: qdf CVdry + sum q CVdry is CVdry up to roundings
      if (!MIX) {
        cva = qdf * CVDRY;
#pragma unroll
        for (int n = 1; n <= 5; ++n)
          if (!((zero >> n) & 1u)) cva = cva + q[n] * CVDRY;
      }
    } else {
      rhog_o = rhog * (1.0 - diffq);
      rho = rhog_o / gsg;
      const double rrhog_o = 1.0 / rhog_o;
#pragma unroll
      for (int n = 1; n <= 5; ++n) q[n] = MIX ? rq[n] * rrhog_o : div_rn(rq[n], rhog_o, rrhog_o);
      qdf = 1.0;
#pragma unroll
      for (int n = 1; n <= 5; ++n) qdf = qdf - q[n];
      cva = CVDRY;
      if (!MIX) {
        cva = qdf * CVDRY;
#pragma unroll
        for (int n = 1; n <= 5; ++n) cva = cva + q[n] * CVDRY;
      }
    }
    rhoge = tem * rhog_o * cva;
    pre = rho * (qdf * RDRY + q[I_QV] * RVAP) * tem;
  }

  P.rhog[i] = rhog_o;
  P.rhoge[i] = rhoge;
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    P.rhogq[iq + (size_t)n * KG] = rq[n];
    P.q[iq + (size_t)n * KG] = q[n];
  }
  P.rho[i] = rho;
  P.tem[i] = tem;
  P.pre[i] = pre;
  P.qd[i] = qd;
  // mp_driver epilogue (mod_mp_driver.cpp:555-612, MP_DIV_NUM = 1)
  P.re_solid[i] = 20.0E-6;
  P.GDCLW[i] = 0.0;
  P.GDCFRC[i] = 0.0;
  if (!interior) {
    P.GPREC[i] = 0.0;
    P.re_liquid[i] = 0.0;
    P.re_cld[i] = 0.0;
  }
  return false;
}

// MIX: the mixed-precision step: the mass and energy fluxes of the
// sedimentation (mass, internal and potential energy) are integrated and their
// divergences summed in FP64 as in the FP64 step; the kinetic-energy and
// momentum fluxes, their sources, the kinetic energies, their tendencies and
// the KIN2EIN correction are FP32; the quotients of the final state use a
// plain reciprocal and its cv sums are lean (every CVW is CVdry); the state
// updates, the internal-energy budget, the thermodynamics and the saturation
// adjustment stay FP64.
//
// OPT: the kernel with the scheme switches (either precision): QI sedimentation (4
// tracers), the KIN2KIN kinetic-energy correction (mod_precip_transport.cpp:
// 1012-1068) and the mixed-phase saturation adjustment (satadjust_all,
// mod_satadjust.cpp:620-769).
template <int COL_TG, class M, bool MIX, bool OPT = false>
__global__ void __launch_bounds__(384, 2) nsw6_column_kernel(Problem P, Consts C) {
  extern __shared__ double smraw[];
  const int G = P.gall, K = P.kall, kmin = P.kmin, kmax = P.kmax;
  constexpr int NSLOT = OPT ? S_COUNT_OPT : S_COUNT;
  constexpr int NROW_MAX = OPT ? 8 : 6;
  const int ntr = OPT ? P.ntr : 3;
  const int nrow = 2 * ntr;
  const bool kin2kin = OPT && C.opt_kin2kin != 0.0;
  const bool ice_adj = OPT && C.opt_expice == 0.0;
  const int l = blockIdx.y;
  const int g0 = blockIdx.x * COL_TG;
  const size_t KG = (size_t)K * G;
  const size_t off = (size_t)l * KG;
  const size_t offq = (size_t)l * NQ * KG;
  const int ncell = K * COL_TG;
  const double dt = P.dt;

  ColumnShared S;
  S.f = smraw;
  S.grid = S.f + (size_t)NSLOT * ncell;
  S.colacc = S.grid + GF_COUNT * K;
  S.bmin = reinterpret_cast<int*>(S.colacc + 6 * COL_TG);
  S.bmax = S.bmin + NROW_MAX * K;
  S.kc = reinterpret_cast<unsigned char*>(S.bmax + NROW_MAX * K);
  const bool tab_smem = !OPT || K <= COL_FMTAB_SMEM_KMAX;
  double* after_kc = reinterpret_cast<double*>(
      (reinterpret_cast<uintptr_t>(S.kc + (size_t)K * COL_TG) + 15) & ~(uintptr_t)15);
  const double* tab = tab_smem ? after_kc : P.fmtab;
  long long* zkey = reinterpret_cast<long long*>(after_kc + (tab_smem ? FM_TABLE_DOUBLES : 0));   // [2][K]: cmp_key of gzh, gzshift
  // MIX: dgz, dgzh, rdgz, rdgzh, afact, bfact, cfact, dfact in FP32
  float* gf = reinterpret_cast<float*>(zkey + 2 * K);
  auto F = [&](int slot) { return S.f + (size_t)slot * ncell; };
  // FP32 views of slots (MIX): the flux source and flux of the FP32 passes,
  // the momentum accumulators and the kinetic energies.  A slot's FP32 view
  // has two halves, [0, ncell) and [ncell, 2 ncell); the thread of cell c
  // owns entries c and ncell + c of each.
  auto FF = [&](int slot) { return reinterpret_cast<float*>(S.f + (size_t)slot * ncell); };

  for (int c = threadIdx.x; c < GF_COUNT * K; c += blockDim.x) S.grid[c] = P.grid[c];
  for (int c = threadIdx.x; c < 2 * K; c += blockDim.x)
    zkey[c] = cmp_key(P.grid[(c < K ? GF_GZH : GF_GZSHIFT) * K + c % K]);
  // MIX: the tile's unit vectors ix, iy, iz, jx, jy, jz in FP32 ([6][COL_TG]);
  // they meet FP32 values only (the velocity components, the momentum tendencies)
  float* uvf = gf + 8 * K;
  if (MIX) {
    const int rows[8] = {GF_DGZ, GF_DGZH, GF_RDGZ, GF_RDGZH, GF_AFACT, GF_BFACT, GF_CFACT, GF_DFACT};
    for (int c = threadIdx.x; c < 8 * K; c += blockDim.x) gf[c] = (float)P.grid[rows[c / K] * K + c % K];
    for (int c = threadIdx.x; c < 6 * COL_TG; c += blockDim.x) {
      const int a = c / COL_TG, g = g0 + c % COL_TG;
      const double* u = a == 0 ? P.ix : a == 1 ? P.iy : a == 2 ? P.iz : a == 3 ? P.jx : a == 4 ? P.jy : P.jz;
      uvf[c] = g < G ? (float)u[(size_t)l * G + g] : 0.0f;
    }
  }
  for (int c = threadIdx.x; c < 6 * COL_TG; c += blockDim.x) S.colacc[c] = 0.0;
  if (tab_smem)
    for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) after_kc[c] = P.fmtab[c];
  __syncthreads();
  const M mth = make_math<M>(tab);
  const double* gzh = S.grid + GF_GZH * K;
  const double* gzs = S.grid + GF_GZSHIFT * K;
  const double* dgz = S.grid + GF_DGZ * K;
  const double* dgzh = S.grid + GF_DGZH * K;
  const double* rdgz = S.grid + GF_RDGZ * K;
  const double* rdgzh = S.grid + GF_RDGZH * K;
  const double* afact = S.grid + GF_AFACT * K;
  const double* bfact = S.grid + GF_BFACT * K;
  const double* cfact = S.grid + GF_CFACT * K;
  const double* dfact = S.grid + GF_DFACT * K;

  // ---- kcell_min/max per level from the region extrema (mod_vadv1d.cpp:316-353)
  for (int c = threadIdx.x; c < nrow * K; c += blockDim.x) {
    const int s = c / K, k = c % K;
    const int half = s / ntr;
    const int mkmin = half ? kmin + 1 : kmin;
    const double* zh = half ? gzs : gzh;
    int bmn = k, bmx = k;
    if (k >= mkmin && k <= kmax) {
      const size_t e = ((size_t)l * nrow + s) * K + k;
      const unsigned long long kx = P.zmax[e], kn = P.zmin[e];
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
            bmn = k2;
            break;
          }
      }
      if (zzmin < 0.0) {
        for (int k2 = k; k2 <= kmax; ++k2)
          if ((zh[k2] <= zh[k] - zzmin) && (zh[k2 + 1] > zh[k] - zzmin)) {
            bmx = k2;
            break;
          }
      }
    }
    S.bmin[c] = bmn;
    S.bmax[c] = bmx;
  }

  // Per-thread values of the half-level metric factors, kept in registers
  // across the passes: every pass gives a thread the same cells
  // c = threadIdx.x + j blockDim.x, j < NJ (NJ covers column_threads()).
  constexpr int NJ = COL_TG == 16 ? 4 : 5;
  double r_rgsh[NJ], r_c2w0[NJ], r_c2w1[NJ];   // gam2h / gsgam2h and C2Wfact at half level k
  // MIX: gam2h / gsgam2h (it scales FP32 sources only) and C2Wfact (they
  // scale the FP32 vertical kinetic energies only) in FP32
  float r_rgshf[NJ], r_c2w0f[NJ], r_c2w1f[NJ];
  const float* aff = gf + 4 * K;   // MIX: afact, bfact, cfact, dfact in FP32
  const float* bff = gf + 5 * K;
  const float* cff = gf + 6 * K;
  const float* dff = gf + 7 * K;

  // ---- metric factors, kinetic energy, zeroed accumulators
  //      (mod_precip_transport.cpp:715-770, cnvvar_rhogkin_in mod_debug.cpp:269-330)
  // MIX keeps these FP32 values in the FP32 halves of slots it uses as FP32:
  //   S_KINH: kinetic energy (horizontal) | rhog (before, then after the transport)
  //   S_KINV: kinetic energy (vertical)   | gam2 / gsgam2 of the cell
  //   S_DKINH: its tendency               | rhoq of the tracer being transported
  //   S_DKINV: its tendency               | rhogw of the half level (before)
  //   S_VI, S_VJ: the velocity components | gsgam2h, gsgam2 of the cell
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int c = threadIdx.x + j * blockDim.x;
    r_rgsh[j] = r_c2w0[j] = r_c2w1[j] = 0.0;
    r_rgshf[j] = r_c2w0f[j] = r_c2w1f[j] = 0.0f;
    if (c >= ncell) continue;
    const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
    for (int s = S_KINH; s <= S_DQG; ++s) {
      if (MIX && (s == S_KINH || s == S_KINV || s == S_DKINH || s == S_DKINV)) {
        FF(s)[c] = 0.0f;
        FF(s)[ncell + c] = 0.0f;
      } else {
        F(s)[c] = 0.0;
      }
    }
    if (OPT) F(S_DQI)[c] = 0.0;
    F(S_RGS)[c] = 0.0;
    if (MIX) {
      FF(S_VI)[c] = FF(S_VI)[ncell + c] = 0.0f;
      FF(S_VJ)[c] = FF(S_VJ)[ncell + c] = 0.0f;
    } else {
      F(S_VI)[c] = 0.0;
      F(S_VJ)[c] = 0.0;
    }
    if (g >= G) continue;
    const size_t i = off + (size_t)k * G + g;
    const size_t ic = (size_t)l * G + g;
    const bool interior = (k >= kmin && k <= kmax);
    // gam2 / gsgam2, afact / gsgam2 and (below) the level above's bfact /
    // gsgam2 from one reciprocal, correctly rounded; the reciprocal waits in
    // S_BASE (free until the transport) for that level
    const double gsg = P.gsgam2[i];
    const double rgsg = 1.0 / gsg;
    if (!MIX) F(S_BASE)[c] = rgsg;
    if (interior) F(S_RGS)[c] = div_rn(P.gam2[i], gsg, rgsg);
    if (MIX) {
      // the velocity components scale FP32 momentum sources only: FP32
      const float vx = (float)P.vx[i], vy = (float)P.vy[i], vz = (float)P.vz[i];
      FF(S_VI)[c] = __fmaf_rn(vz, uvf[2 * COL_TG + gx], __fmaf_rn(vy, uvf[1 * COL_TG + gx], __fmul_rn(vx, uvf[gx])));
      FF(S_VJ)[c] =
          __fmaf_rn(vz, uvf[5 * COL_TG + gx], __fmaf_rn(vy, uvf[4 * COL_TG + gx], __fmul_rn(vx, uvf[3 * COL_TG + gx])));
      const float gsgf = (float)gsg, ghf = (float)P.gsgam2h[i], rhogf = (float)P.rhog[i];
      FF(S_VI)[ncell + c] = ghf;
      FF(S_VJ)[ncell + c] = gsgf;
      FF(S_KINH)[ncell + c] = rhogf;
      if (interior) {
        FF(S_KINV)[ncell + c] = (float)F(S_RGS)[c];
        FF(S_KINH)[c] = kin_h_f((float)P.rhogvx[i], (float)P.rhogvy[i], (float)P.rhogvz[i], rhogf);
      }
      if (k >= kmin + 1 && k <= kmax) {
        r_c2w0f[j] = __fmul_rn(__fdiv_rn(aff[k], gsgf), ghf);
        r_rgshf[j] = __fdiv_rn((float)P.gam2h[i], ghf);
      }
      continue;
    }
    const double vx = P.vx[i], vy = P.vy[i], vz = P.vz[i];
    F(S_VI)[c] = vx * P.ix[ic] + vy * P.iy[ic] + vz * P.iz[ic];
    F(S_VJ)[c] = vx * P.jx[ic] + vy * P.jy[ic] + vz * P.jz[ic];
    if (interior) {
      const double rvx = P.rhogvx[i], rvy = P.rhogvy[i], rvz = P.rhogvz[i];
      F(S_KINH)[c] = 0.5 * (rvx * rvx + rvy * rvy + rvz * rvz) / P.rhog[i];
    }
    if (k >= kmin + 1 && k <= kmax) {
      r_c2w0[j] = div_rn(afact[k], gsg, rgsg) * P.gsgam2h[i];
      r_rgsh[j] = P.gam2h[i] / P.gsgam2h[i];
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int c = threadIdx.x + j * blockDim.x;
    if (c >= ncell) continue;
    const int k = c / COL_TG, g = g0 + c % COL_TG;
    if (g >= G || k < kmin + 1 || k > kmax) continue;
    const size_t i = off + (size_t)k * G + g;
    if (MIX) {
      const float c2w1 = __fmul_rn(__fdiv_rn(bff[k], FF(S_VJ)[ncell + c - COL_TG]), FF(S_VI)[ncell + c]);
      const float rw = (float)P.rhogw[i];
      FF(S_DKINV)[ncell + c] = rw;
      FF(S_KINV)[c] = kin_v_f(rw, r_c2w0f[j], c2w1, FF(S_KINH)[ncell + c], FF(S_KINH)[ncell + c - COL_TG]);
      r_c2w1f[j] = c2w1;
      continue;
    }
    const double c2w0 = r_c2w0[j];
    const double c2w1 = div_rn(bfact[k], P.gsgam2[i - G], F(S_BASE)[c - COL_TG]) * P.gsgam2h[i];
    const double rw = P.rhogw[i];
    F(S_KINV)[c] = 0.5 * (rw * rw) / (c2w0 * P.rhog[i] + c2w1 * P.rhog[i - G]);
    r_c2w1[j] = c2w1;
  }
  __syncthreads();

  // ---- sedimentation of QR, QS, QG (mod_precip_transport.cpp:767-955)
  // tracers in the reference's order (QI sediments with "4WATER")
  for (int t = 0; t < ntr; ++t) {
    const int nq = ntr == 4 ? (t == 0 ? I_QR : t == 1 ? I_QI : t == 2 ? I_QS : I_QG) : (t == 0 ? I_QR : t == 1 ? I_QS : I_QG);
    const int dqs_slot = nq == I_QR ? S_DQR : nq == I_QS ? S_DQS : nq == I_QG ? S_DQG : S_DQI;
    // departure distances of this region: [2 ntr][K][G] rows t (full) and ntr + t (half)
    const double* zdis0 = P.zdis + ((size_t)l * nrow + t) * KG;
    const double* zdis0h = P.zdis + ((size_t)l * nrow + ntr + t) * KG;
    const int* bmn_f = S.bmin + t * K;
    const int* bmx_f = S.bmax + t * K;
    const int* bmn_h = S.bmin + (ntr + t) * K;
    const int* bmx_h = S.bmax + (ntr + t) * K;
    const double* rhogq_n = P.rhogq + offq + (size_t)nq * KG;
    const double* q_n = P.q + offq + (size_t)nq * KG;

    // departure cells (full levels) and rhoq = rhogq * rgs, which is also
    // the source of the first flux (the mass flux)
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
      const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
      if (g >= G) {
        F(S_RHOF)[c] = 0.0;
        continue;
      }
      const size_t i = (size_t)k * G + g;
      const double b = rhogq_n[i] * F(S_RGS)[c];
      F(S_BASE)[c] = b;
      F(S_RHOF)[c] = b;
      if (k >= kmin && k <= kmax)
        S.kc[c] = (unsigned char)departure_cell(gzh, zkey, k, zdis0[i], bmn_f[k], bmx_f[k], kmin, kmax);
    }
    __syncthreads();

    // flux source: q, e, phi, kin_h, u, v (mod_precip_transport.cpp:776-808)
    auto source = [&](int f, int c) {
      const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
      if (MIX && f >= 3) {
        // FP32 sources of the kinetic-energy and momentum fluxes; rhoq in FP32
        // is formed once, with the first of them
        float r = 0.0f;
        if (g < G) {
          if (f == 3) {
            FF(S_DKINH)[ncell + c] = (float)F(S_BASE)[c];
            r = __fmul_rn(__fmul_rn((float)q_n[(size_t)k * G + g], FF(S_KINV)[ncell + c]), FF(S_KINH)[c]);
          } else {
            r = __fmul_rn(FF(S_DKINH)[ncell + c], f == 4 ? FF(S_VI)[c] : FF(S_VJ)[c]);
          }
        }
        FF(S_RHOF)[c] = r;
        return;
      }
      double r = 0.0;
      if (g < G) {
        const size_t i = off + (size_t)k * G + g;
        const double b = F(S_BASE)[c];
        switch (f) {
          case 0: r = b; break;
          case 1: r = b * CVDRY * P.tem[i]; break;
          case 2: r = b * GRAV * P.z[i]; break;
          case 3: r = q_n[i - off] * F(S_RGS)[c] * F(S_KINH)[c]; break;
          case 4: r = b * F(S_VI)[c]; break;
          default: r = b * F(S_VJ)[c]; break;
        }
      }
      F(S_RHOF)[c] = r;
    };
    // flux divergence and surface fluxes (mod_precip_transport.cpp:782-842,
    // 900-954); the quotients by dt are the correctly rounded ones, formed
    // from 1/dt
    auto divergence = [&](int f, int c) {
      const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
      if (g >= G || k < kmin || k > kmax) return;
      const double fk = F(S_F)[c], fk1 = F(S_F)[c + COL_TG];
      const double d = (fk1 - fk) * rdgz[k];
      switch (f) {
        case 0:
          F(dqs_slot)[c] = -d;
          if (nq == I_QR) P.GPREC[off + (size_t)k * G + g] = plus_zero(div_rn(-fk, dt, P.rdt));
          break;
        case 1: F(S_DRHOE)[c] = F(S_DRHOE)[c] - d; break;
        case 2: F(S_DRHOPHI)[c] = F(S_DRHOPHI)[c] - d; break;
        case 3: F(S_DKINH)[c] = F(S_DKINH)[c] - d; break;
        case 4: F(S_DRHOGU)[c] = F(S_DRHOGU)[c] - d; break;
        default: F(S_DRHOGV)[c] = F(S_DRHOGV)[c] - d; break;
      }
      if (k == kmin) {
        double* acc = S.colacc;
        const double fdt = div_rn(fk, dt, P.rdt);
        switch (f) {
          case 0:
            if (nq == I_QR) {
              acc[0 * COL_TG + gx] = acc[0 * COL_TG + gx] - fdt;
            } else {
              acc[1 * COL_TG + gx] = acc[1 * COL_TG + gx] - fdt;
              acc[2 * COL_TG + gx] = acc[2 * COL_TG + gx] + div_rn(fk * LHF0, dt, P.rdt);
            }
            break;
          case 1: acc[3 * COL_TG + gx] = acc[3 * COL_TG + gx] - fdt; break;
          case 2: acc[4 * COL_TG + gx] = acc[4 * COL_TG + gx] - fdt; break;
          case 3: acc[5 * COL_TG + gx] = acc[5 * COL_TG + gx] - fdt; break;
          default: break;
        }
      }
    };
    // the divergence of flux f and the source of flux f + 1 share a pass (the
    // source of flux 0 is rhoq, written above)
    if (!MIX) {
      for (int f = 0; f < 6; ++f) {
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          double fl = 0.0;
          if (g < G && k >= kmin && k <= kmax)
            fl = flux_integral<COL_TG>(F(S_RHOF) + gx, dgz, k, S.kc[c], zdis0[(size_t)k * G + g], bmn_f[k], bmx_f[k]);
          F(S_F)[c] = fl;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          divergence(f, c);
          if (f + 1 < 6) source(f + 1, c);
        }
        __syncthreads();
      }
    } else {
      // the mass and energy fluxes (mass, internal and potential energy) as
      // in the FP64 step; the kinetic-energy and momentum ones, their sources
      // and tendencies in FP32
      const float* rf = FF(S_RHOF);
      float* ff = FF(S_F);
      const float* dgzf = gf;
      const float* rdgzf = gf + 2 * K;
      for (int f = 0; f < 3; ++f) {
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          double fl = 0.0;
          if (g < G && k >= kmin && k <= kmax)
            fl = flux_integral<COL_TG>(F(S_RHOF) + gx, dgz, k, S.kc[c], zdis0[(size_t)k * G + g], bmn_f[k], bmx_f[k]);
          F(S_F)[c] = fl;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          divergence(f, c);
          source(f + 1, c);
          if (f == 2) {
            // the FP32 departure distance of the three FP32 fluxes, converted once,
            // in the upper half of the slot whose lower half now holds FP32 sources
            const int k = c / COL_TG, g = g0 + c % COL_TG;
            if (g < G && k >= kmin && k <= kmax) FF(S_RHOF)[ncell + c] = (float)zdis0[(size_t)k * G + g];
          }
        }
        __syncthreads();
      }
      for (int f = 3; f < 6; ++f) {
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          float fl = 0.0f;
          if (g < G && k >= kmin && k <= kmax)
            fl = flux_integral_f<COL_TG>(rf + gx, dgzf, k, S.kc[c], rf[ncell + c], bmn_f[k], bmx_f[k]);
          ff[c] = fl;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          if (g < G && k >= kmin && k <= kmax) {
            const float d = (ff[c + COL_TG] - ff[c]) * rdgzf[k];
            switch (f) {
              case 3: FF(S_DKINH)[c] = FF(S_DKINH)[c] - d; break;
              case 4: FF(S_DRHOGU)[c] = FF(S_DRHOGU)[c] - d; break;
              default: FF(S_DRHOGV)[c] = FF(S_DRHOGV)[c] - d; break;
            }
            // the kinetic energy reaching the ground (precip_rhokin)
            if (k == kmin && f == 3)
              S.colacc[5 * COL_TG + gx] = S.colacc[5 * COL_TG + gx] - div_rn((double)ff[c], dt, P.rdt);
          }
          if (f + 1 < 6) source(f + 1, c);
        }
        __syncthreads();
      }
    }

    // half levels: departure cells and qh (mod_precip_transport.cpp:845-882)
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int c = threadIdx.x + j * blockDim.x;
      if (c >= ncell) continue;
      const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
      const bool hv = g < G && k >= kmin + 1 && k <= kmax;
      if (hv)
        S.kc[c] = (unsigned char)departure_cell(gzs, zkey + K, k, zdis0h[(size_t)k * G + g], bmn_h[k], bmx_h[k], kmin + 1,
                                                kmax);
      if (MIX) {
        // qh scales the FP32 sources of the two half-level fluxes only: FP32
        float qh = 0.0f;
        if (hv) qh = 0.5f * (float(q_n[(size_t)k * G + g]) + float(q_n[(size_t)(k - 1) * G + g])) * r_rgshf[j];
        FF(S_BASE)[c] = qh;
        FF(S_RHOF)[c] = __fmul_rn(qh, FF(S_KINV)[c]);
        // the half levels' FP32 departure distance, converted once (upper half)
        if (hv) FF(S_RHOF)[ncell + c] = (float)zdis0h[(size_t)k * G + g];
      } else {
        double qh = 0.0;
        if (hv) qh = 0.5 * (q_n[(size_t)k * G + g] + q_n[(size_t)(k - 1) * G + g]) * r_rgsh[j];
        F(S_BASE)[c] = qh;
        F(S_RHOF)[c] = qh * F(S_KINV)[c];
      }
    }
    __syncthreads();
    for (int w = 0; w < 2; ++w) {
      if (MIX && w == 0) {
        // vertical kinetic energy in FP32 and its FP32 tendency; the pass also
        // forms the FP32 source of momentum w
        const float* rf = FF(S_RHOF);
        float* ff = FF(S_F);
        const float* dgzhf = gf + K;
        const float* rdgzhf = gf + 3 * K;
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          float fl = 0.0f;
          if (g < G && k >= kmin + 1 && k <= kmax)
            fl = flux_integral_f<COL_TG>(rf + gx, dgzhf, k, S.kc[c], rf[ncell + c], bmn_h[k], bmx_f[k]);
          ff[c] = fl;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          float r = 0.0f;
          if (g < G && k >= kmin + 1 && k <= kmax) {
            FF(S_DKINV)[c] = FF(S_DKINV)[c] - (ff[c] - ff[c - COL_TG]) * rdgzhf[k];
            r = FF(S_BASE)[c] * FF(S_DKINV)[ncell + c];   // rhogw before the transport, in FP32
          }
          FF(S_RHOF)[c] = r;
        }
        __syncthreads();
        continue;
      }
      if (MIX && w == 1) {
        // momentum w in FP32 (its source was written as FP32 by the w = 0 pass)
        const float* rf = FF(S_RHOF);
        float* ff = FF(S_F);
        float* acc = FF(S_DRHOGW);
        const float* dgzhf = gf + K;
        const float* rdgzhf = gf + 3 * K;
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          float fl = 0.0f;
          if (g < G && k >= kmin + 1 && k <= kmax)
            fl = flux_integral_f<COL_TG>(rf + gx, dgzhf, k, S.kc[c], rf[ncell + c], bmn_h[k], bmx_f[k]);
          ff[c] = fl;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
          const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
          if (g < G && k >= kmin + 1 && k <= kmax) acc[c] = acc[c] - (ff[c] - ff[c - COL_TG]) * rdgzhf[k];
        }
        __syncthreads();
        continue;
      }
      // vertical kinetic energy (w = 0) and momentum w (w = 1); the reference
      // passes the full-level kcell_max as the upper bound (:890, :892)
      for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
        const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
        double fl = 0.0;
        if (g < G && k >= kmin + 1 && k <= kmax)
          fl = flux_integral<COL_TG>(F(S_RHOF) + gx, dgzh, k, S.kc[c], zdis0h[(size_t)k * G + g], bmn_h[k], bmx_f[k]);
        F(S_F)[c] = fl;
      }
      __syncthreads();
      for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
        const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
        if (g < G && k >= kmin + 1 && k <= kmax) {
          const double d = (F(S_F)[c] - F(S_F)[c - COL_TG]) * rdgzh[k];
          if (w == 0) F(S_DKINV)[c] = F(S_DKINV)[c] - d;
          else F(S_DRHOGW)[c] = F(S_DRHOGW)[c] - d;
        }
        if (w == 0) {
          double r = 0.0;
          if (g < G && k >= kmin + 1 && k <= kmax) r = F(S_BASE)[c] * P.rhogw[off + (size_t)k * G + g];
          if (MIX) FF(S_RHOF)[c] = (float)r;
          else F(S_RHOF)[c] = r;
        }
      }
      __syncthreads();
    }
  }

  // ---- apply the tendencies (mod_precip_transport.cpp:956-989)
  for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
    const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
    if (g >= G) continue;
    const size_t i = off + (size_t)k * G + g;
    const size_t ic = (size_t)l * G + g;
    const size_t iq = offq + (size_t)k * G + g;
    const double dqr = F(S_DQR)[c], dqs = F(S_DQS)[c], dqg = F(S_DQG)[c];
    double rhoge = P.rhoge[i] + F(S_DRHOE)[c] + F(S_DRHOPHI)[c];
    if (MIX) {
      FF(S_KINH)[c] = FF(S_KINH)[c] + FF(S_DKINH)[c];
      FF(S_KINV)[c] = FF(S_KINV)[c] + FF(S_DKINV)[c];
    } else {
      F(S_KINH)[c] = F(S_KINH)[c] + F(S_DKINH)[c];
      F(S_KINV)[c] = F(S_KINV)[c] + F(S_DKINV)[c];
    }
    if (MIX) {
      // the FP32 momentum tendencies along the FP32 unit vectors, added to the FP64 state
      const float du = FF(S_DRHOGU)[c], dv = FF(S_DRHOGV)[c];
      P.rhogvx[i] = P.rhogvx[i] + (double)__fmaf_rn(dv, uvf[3 * COL_TG + gx], __fmul_rn(du, uvf[gx]));
      P.rhogvy[i] = P.rhogvy[i] + (double)__fmaf_rn(dv, uvf[4 * COL_TG + gx], __fmul_rn(du, uvf[1 * COL_TG + gx]));
      P.rhogvz[i] = P.rhogvz[i] + (double)__fmaf_rn(dv, uvf[5 * COL_TG + gx], __fmul_rn(du, uvf[2 * COL_TG + gx]));
    } else {
      const double du = F(S_DRHOGU)[c], dv = F(S_DRHOGV)[c];
      P.rhogvx[i] = P.rhogvx[i] + du * P.ix[ic] + dv * P.jx[ic];
      P.rhogvy[i] = P.rhogvy[i] + du * P.iy[ic] + dv * P.jy[ic];
      P.rhogvz[i] = P.rhogvz[i] + du * P.iz[ic] + dv * P.jz[ic];
    }
    const double rw = P.rhogw[i] + (MIX ? (double)FF(S_DRHOGW)[c] : F(S_DRHOGW)[c]);
    P.rhogw[i] = rw;
    if (!MIX) F(S_DRHOGW)[c] = rw;   // MIX: the FP32 view of this slot is still being read
    // tracers in order QV..QG; QV, QC and QI add exact zeros (plus_zero: the addition of +0 on the integer pipe)
    double rhog = P.rhog[i];
    const double zz = P.z[i];
    P.rhogq[iq + (size_t)I_QV * KG] = plus_zero(P.rhogq[iq + (size_t)I_QV * KG]);
    P.rhogq[iq + (size_t)I_QC * KG] = plus_zero(P.rhogq[iq + (size_t)I_QC * KG]);
    P.rhogq[iq + (size_t)I_QR * KG] = P.rhogq[iq + (size_t)I_QR * KG] + dqr;
    rhog = rhog + dqr;
    rhoge = rhoge - dqr * GRAV * zz;
    if (OPT && ntr == 4) {
      const double dqi = F(S_DQI)[c];
      P.rhogq[iq + (size_t)I_QI * KG] = P.rhogq[iq + (size_t)I_QI * KG] + dqi;
      rhog = rhog + dqi;
      rhoge = rhoge - dqi * GRAV * zz;
    } else {
      P.rhogq[iq + (size_t)I_QI * KG] = plus_zero(P.rhogq[iq + (size_t)I_QI * KG]);
    }
    P.rhogq[iq + (size_t)I_QS * KG] = P.rhogq[iq + (size_t)I_QS * KG] + dqs;
    rhog = rhog + dqs;
    rhoge = rhoge - dqs * GRAV * zz;
    P.rhogq[iq + (size_t)I_QG * KG] = P.rhogq[iq + (size_t)I_QG * KG] + dqg;
    rhog = rhog + dqg;
    rhoge = rhoge - dqg * GRAV * zz;
    P.rhog[i] = rhog;
    P.rhoge[i] = rhoge;
    F(S_RHOF)[c] = rhog;
    if (MIX) FF(S_KINH)[ncell + c] = (float)rhog;   // rhog after the transport, for the FP32 kinetic energies
  }
  __syncthreads();

  // ---- KIN2KIN (mod_precip_transport.cpp:1012-1068), with the switch: the
  //      momentum is rescaled so that the kinetic energy carried by the
  //      transport is kept, horizontal on [kmin, kmax], vertical on
  //      [kmin, kmax+1] (where the carried energy is zero at kmin and kmax+1)
  if (kin2kin) {
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
      const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
      if (g >= G || k < kmin || k > kmax + 1) continue;
      const size_t i = off + (size_t)k * G + g;
      const double rhog = F(S_RHOF)[c];
      if (k <= kmax) {
        const double kin_h0 = (MIX ? (double)FF(S_KINH)[c] : F(S_KINH)[c]) / rhog;
        double vx_t = P.rhogvx[i] / rhog, vy_t = P.rhogvy[i] / rhog, vz_t = P.rhogvz[i] / rhog;
        const double kin_h = 0.5 * (vx_t * vx_t + vy_t * vy_t + vz_t * vz_t);
        if (kin_h > 1.0E-20) {
          const double r = sqrt(fabs(kin_h0 / kin_h));
          vx_t = vx_t * r;
          vy_t = vy_t * r;
          vz_t = vz_t * r;
        }
        P.rhogvx[i] = vx_t * rhog;
        P.rhogvy[i] = vy_t * rhog;
        P.rhogvz[i] = vz_t * rhog;
      }
      const double c2w0 = afact[k] / P.gsgam2[i] * P.gsgam2h[i];
      const double c2w1 = bfact[k] / P.gsgam2[i - G] * P.gsgam2h[i];
      const double rhogh = c2w0 * rhog + c2w1 * F(S_RHOF)[c - COL_TG];
      const double kin_v0 = (MIX ? (double)FF(S_KINV)[c] : F(S_KINV)[c]) / rhogh;
      double w_t = P.rhogw[i] / rhogh;
      const double kin_v = 0.5 * (w_t * w_t);
      if (kin_v > 1.0E-20) w_t = w_t * sqrt(fabs(kin_v0 / kin_v));
      P.rhogw[i] = w_t * rhogh;
    }
  }

  // ---- KIN2EIN (mod_precip_transport.cpp:991-1011): tmp2 and the vertical
  //      kinetic energy of the updated state
  //      (and, in the reference configuration's kernel, the metric factors
  //      W2Cfact of each interior cell for the final pass, in the dead slots
  //      S_DRHOGW / S_DRHOGV, read after rw)
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int c = threadIdx.x + j * blockDim.x;
    if (c >= ncell || kin2kin) continue;
    const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
    if (MIX) {
      // FP32: the change of the vertical kinetic energy of half level k by
      // the transport, (KINV + its tendency) - the energy of the updated
      // state, in the FP32 half of S_DRHOPHI (zero where there is none), and
      // W2Cfact of the interior cells in the two halves of S_DRHOE
      float dkv = 0.0f;
      if (g < G && k >= kmin + 1 && k <= kmax) {
        const size_t i = off + (size_t)k * G + g;
        dkv = FF(S_KINV)[c] - kin_v_f((float)P.rhogw[i], r_c2w0f[j], r_c2w1f[j], FF(S_KINH)[ncell + c],
                                      FF(S_KINH)[ncell + c - COL_TG]);
      }
      FF(S_DRHOPHI)[c] = dkv;
      if (g < G && k >= kmin && k <= kmax) {
        const float gsgf = FF(S_VJ)[ncell + c], ghu = FF(S_VI)[ncell + c + COL_TG];
        FF(S_DRHOE)[c] = __fdiv_rn(__fmul_rn(cff[k], gsgf), ghu);
        FF(S_DRHOE)[ncell + c] = __fdiv_rn(__fmul_rn(dff[k], gsgf), ghu);
      }
      continue;
    }
    F(S_DRHOE)[c] = 0.0;
    F(S_DRHOPHI)[c] = 0.0;
    if (g >= G) continue;
    const size_t i = off + (size_t)k * G + g;
    const bool hk = (k >= kmin + 1 && k <= kmax);
    const double rw = hk ? F(S_DRHOGW)[c] : 0.0;
    if (k >= kmin && k <= kmax) {
      const double gh = P.gsgam2h[i + G], rgh = 1.0 / gh;
      const double w2c0 = div_rn(cfact[k] * P.gsgam2[i], gh, rgh);
      const double w2c1 = div_rn(dfact[k] * P.gsgam2[i], gh, rgh);
      F(S_DRHOE)[c] = F(S_KINH)[c] + (w2c0 * F(S_KINV)[c + COL_TG] + w2c1 * F(S_KINV)[c]);
      if (!OPT) {
        F(S_DRHOGW)[c] = w2c0;
        F(S_DRHOGV)[c] = w2c1;
      }
    }
    if (hk) F(S_DRHOPHI)[c] = 0.5 * (rw * rw) / (r_c2w0[j] * F(S_RHOF)[c] + r_c2w1[j] * F(S_RHOF)[c - COL_TG]);
  }
  __syncthreads();

  // ---- per cell: KIN2EIN, final thermodynamics, saturation adjustment,
  //      negative filter, outputs.  The saturation-adjustment Newton
  //      iteration runs only in saturated cells, a few percent of them; a
  //      tile's would share one warp, which issues one FP64 instruction per
  //      64 cycles where the SM issues one per 19.  So the saturated cells are
  //      left as they are (rhoge after KIN2EIN stored), listed, and finished
  //      by nsw6_satadj_kernel, whose warps are full and fill every SM.
  __shared__ int nqueue;
  __shared__ unsigned qbase;
  if (threadIdx.x == 0) nqueue = 0;
  __syncthreads();
  const float lovr_f = float(C.LovR_liq);
  int* qcell = reinterpret_cast<int*>(F(S_BASE));   // the tile's saturated cells (S_BASE is dead by now)
  for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
    const int k = c / COL_TG, gx = c % COL_TG, g = g0 + gx;
    if (g >= G) continue;
    const size_t i = off + (size_t)k * G + g;
    const bool interior = (k >= kmin && k <= kmax);
    const double rhog = F(S_RHOF)[c];
    // Quotients by a shared denominator are formed from one reciprocal with a
    // Markstein correction step (div_rn): correctly rounded, as the reference's
    // divisions, at a third of the cost.
    const double rrhog = 1.0 / rhog;
    double rhoge = P.rhoge[i];
    if (MIX && interior && !kin2kin) {
      // FP32 kinetic energies: the horizontal energy after the transport
      // against before (with its tendency), the vertical energies' changes
      // weighted by W2Cfact; their sum enters the FP64 internal energy
      const float kh = kin_h_f((float)P.rhogvx[i], (float)P.rhogvy[i], (float)P.rhogvz[i], FF(S_KINH)[ncell + c]);
      const float dke = (FF(S_KINH)[c] - kh) +
                        __fmaf_rn(FF(S_DRHOE)[c], FF(S_DRHOPHI)[c + COL_TG],
                                  __fmul_rn(FF(S_DRHOE)[ncell + c], FF(S_DRHOPHI)[c]));
      rhoge = rhoge + (double)dke;
      P.rhoge[i] = rhoge;   // a saturated cell's adjustment starts from here (final_cell overwrites the rest)
    } else if (interior && !kin2kin) {
      const double rvx = P.rhogvx[i], rvy = P.rhogvy[i], rvz = P.rhogvz[i];
      const double tmp_h = div_rn(0.5 * (rvx * rvx + rvy * rvy + rvz * rvz), rhog, rrhog);
      double w2c0, w2c1;
      if (!OPT) {
        w2c0 = F(S_DRHOGW)[c];
        w2c1 = F(S_DRHOGV)[c];
      } else {
        const double gh = P.gsgam2h[i + G], rgh = 1.0 / gh;
        w2c0 = div_rn(cfact[k] * P.gsgam2[i], gh, rgh);
        w2c1 = div_rn(dfact[k] * P.gsgam2[i], gh, rgh);
      }
      const double tmp = tmp_h + (w2c0 * F(S_DRHOPHI)[c + COL_TG] + w2c1 * F(S_DRHOPHI)[c]);
      rhoge = rhoge + (F(S_DRHOE)[c] - tmp);
      P.rhoge[i] = rhoge;   // a saturated cell's adjustment starts from here (final_cell overwrites the rest)
    }
    if (final_cell<M, MIX, OPT>(P, C, mth, ice_adj, lovr_f, i, offq + (size_t)k * G + g, KG, interior, rhog, rrhog,
                                rhoge, false, k, g, l))
      qcell[atomicAdd(&nqueue, 1)] = c;
    if (k == kmin) {
      const size_t ic = (size_t)l * G + g;
      const size_t r0 = (size_t)l * G + g, r1 = P.prec_ld + r0;
      const double* acc = S.colacc;
      P.precip[r0] = plus_zero(acc[0 * COL_TG + gx]);
      P.precip[r1] = plus_zero(acc[1 * COL_TG + gx]);
      P.iso1[r0] = 0.0;
      P.iso1[r1] = 0.0;
      P.iso2[r0] = 0.0;
      P.iso2[r1] = 0.0;
      P.precip_lh_heat[ic] = plus_zero(acc[2 * COL_TG + gx]);
      P.precip_rhoe[ic] = plus_zero(acc[3 * COL_TG + gx]);
      P.precip_rhophi[ic] = plus_zero(acc[4 * COL_TG + gx]);
      P.precip_rhokin[ic] = plus_zero(acc[5 * COL_TG + gx]);
    }
  }
  __syncthreads();
  // the tile's saturated cells join the list (satq[0] counts them)
  if (threadIdx.x == 0) qbase = nqueue > 0 ? atomicAdd(P.satq, (unsigned)nqueue) : 0u;
  __syncthreads();
  for (int e = threadIdx.x; e < nqueue; e += blockDim.x) {
    const int c = qcell[e];
    P.satq[1 + qbase + e] = (unsigned)(off + (size_t)(c / COL_TG) * G + g0 + c % COL_TG);
  }
}

// ------------------------------------------------------------------ kernel 3
// The saturated cells the column kernel listed (P.satq): the cell's state
// after KIN2EIN is formed again exactly as there, the saturation-adjustment
// Newton iteration runs and the cell is finished (final_cell).  One thread per
// cell, grid-stride over the list, whose length only the device knows.
constexpr int SAT_THREADS = 128;
constexpr int SAT_BLOCKS = 152 * 8;

template <class M, bool MIX, bool OPT>
__global__ void __launch_bounds__(SAT_THREADS) nsw6_satadj_kernel(Problem P, Consts C) {
  __shared__ double tab[FM_TABLE_DOUBLES];
  const unsigned n = P.satq[0];
  if (n == 0) return;
  for (int t = threadIdx.x; t < FM_TABLE_DOUBLES; t += blockDim.x) tab[t] = P.fmtab[t];
  __syncthreads();
  const M mth = make_math<M>(tab);
  const int G = P.gall;
  const size_t KG = (size_t)P.kall * G;
  const bool ice_adj = OPT && C.opt_expice == 0.0;
  const float lovr_f = float(C.LovR_liq);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const size_t i = P.satq[1 + e];
    const int l = (int)(i / KG);
    const size_t r = i - (size_t)l * KG;
    const int k = (int)(r / G), g = (int)(r - (size_t)k * G);
    const double rhog = P.rhog[i];
    final_cell<M, MIX, OPT>(P, C, mth, ice_adj, lovr_f, i, (size_t)l * NQ * KG + r, KG, true, rhog, 1.0 / rhog,
                            P.rhoge[i], true, k, g, l);
  }
}

// ------------------------------------------------------------------ math check
// Evaluates the step's table-driven transcendentals on n inputs:
// fn 0 exp(x), 1 log(x), 2 pow(x, y).
__global__ void nsw6_math_kernel(int fn, const double* x, const double* y, double* out, int n, const double* fmtab) {
  __shared__ double tab[FM_TABLE_DOUBLES];
  for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = fmtab[c];
  __syncthreads();
  const FastMath m = make_math<FastMath>(tab);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = x[i];
    out[i] = fn == 0 ? m.exp(v) : fn == 1 ? m.log(v) : m.pow(v, y[i]);
  }
}

cudaError_t launch_math(int fn, const double* x, const double* y, double* out, int n, const double* fmtab,
                        cudaStream_t stream) {
  const int blocks = n <= 0 ? 1 : (n + 255) / 256 > 1024 ? 1024 : (n + 255) / 256;
  nsw6_math_kernel<<<blocks, 256, 0, stream>>>(fn, x, y, out, n, fmtab);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ launchers
size_t cell_smem_bytes(int K, bool mixed, bool opt) {
  const size_t vts = mixed ? cell_vts_doubles<float>(K, opt ? 4 : 3) : cell_vts_doubles<double>(K, opt ? 4 : 3);
  const size_t staged = (!opt || K <= CELL_SMEM_KMAX) ? (size_t)GF_COUNT * K + FM_TABLE_DOUBLES : 0;
  // fall speeds, grid, tables, the FP32 reciprocal rows, the cell order and keys
  return sizeof(double) * (vts + staged) + sizeof(float) * 4 * K +
         (sizeof(unsigned short) + 1) * (size_t)(K - 2) * CELL_TG + 16 +
         (mixed ? sizeof(float) : sizeof(double)) * (size_t)K * CELL_TG;
}

int column_tile(int K) { return K <= 64 ? 16 : 8; }

size_t column_smem_bytes(int K, bool opt) {
  const int TG = column_tile(K);
  const size_t nslot = opt ? S_COUNT_OPT : S_COUNT;
  const size_t nrow = opt ? 8 : 6;
  const size_t ntab = (!opt || K <= COL_FMTAB_SMEM_KMAX) ? FM_TABLE_DOUBLES : 0;
  return sizeof(double) * (nslot * K * TG + GF_COUNT * K + 6 * TG + ntab) +
         sizeof(int) * 2 * nrow * K + (size_t)K * TG + 16 + sizeof(long long) * 2 * K + sizeof(float) * 8 * K +
         sizeof(float) * 6 * TG;
}

int column_threads(int K) {
  const int ncell = K * column_tile(K);
  const int passes = (ncell + 383) / 384;
  int per = (ncell + passes - 1) / passes;
  per = (per + 31) / 32 * 32;
  return per > 384 ? 384 : per;
}

cudaError_t launch_prepare();

// The cell kernel alone (FP64): used on a copy of a state to obtain the
// region extrema of the departure distances for the derivative kernels.
cudaError_t launch_cell_only(const Problem& P, const Consts& C, cudaStream_t stream) {
  const size_t nkey = (size_t)P.lall * 2 * P.ntr * P.kall;
  cudaError_t e = cudaMemsetAsync(P.zmax, 0x00, nkey * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(P.zmin, 0xff, nkey * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  e = launch_prepare();
  if (e != cudaSuccess) return e;
  dim3 g1((P.gall + CELL_TG - 1) / CELL_TG, P.lall);
  if (P.opt)
    nsw6_cell_kernel<FastMath, double, true><<<g1, CELL_THREADS, cell_smem_bytes(P.kall, false, true), stream>>>(P, C);
  else
    nsw6_cell_kernel<FastMath, double><<<g1, CELL_THREADS, cell_smem_bytes(P.kall, false, false), stream>>>(P, C);
  return cudaGetLastError();
}

// Raises a kernel's dynamic shared-memory limit to what the device allows a
// block beside the kernel's own static shared memory.
template <class Kernel>
static cudaError_t raise_smem_limit(Kernel k, int optin) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes);
}

// Opt-in shared-memory limits of the step kernels (once per process; before
// any stream capture of a step).
cudaError_t launch_prepare() {
  static cudaError_t done = cudaErrorNotReady;
  if (done == cudaErrorNotReady) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const cudaError_t r[] = {
        e,
        raise_smem_limit(nsw6_cell_kernel<FastMath, double>, optin),
        raise_smem_limit(nsw6_cell_kernel<LibMath, double>, optin),
        raise_smem_limit(nsw6_cell_kernel<FloatMath, float>, optin),
        raise_smem_limit(nsw6_cell_kernel<FastMath, double, true>, optin),
        raise_smem_limit(nsw6_column_kernel<16, FastMath, false, true>, optin),
        raise_smem_limit(nsw6_column_kernel<8, FastMath, false, true>, optin),
        raise_smem_limit(nsw6_column_kernel<16, FastMath, false>, optin),
        raise_smem_limit(nsw6_column_kernel<8, FastMath, false>, optin),
        raise_smem_limit(nsw6_column_kernel<16, LibMath, false>, optin),
        raise_smem_limit(nsw6_column_kernel<8, LibMath, false>, optin),
        raise_smem_limit(nsw6_column_kernel<16, FastMath, true>, optin),
        raise_smem_limit(nsw6_column_kernel<8, FastMath, true>, optin),
        raise_smem_limit(nsw6_cell_kernel<FloatMath, float, true>, optin),
        raise_smem_limit(nsw6_column_kernel<16, FastMath, true, true>, optin),
        raise_smem_limit(nsw6_column_kernel<8, FastMath, true, true>, optin)};
    done = cudaSuccess;
    for (cudaError_t x : r)
      if (x != cudaSuccess) done = x;
  }
  return done;
}

// before_column (may be null): an event the column kernel waits for (inputs
// that only it reads may still be arriving while the cell kernel runs).
cudaError_t launch_step(const Problem& P, const Consts& C, cudaStream_t stream, cudaEvent_t* ev,
                        cudaEvent_t before_column) {
  const size_t nkey = (size_t)P.lall * 2 * P.ntr * P.kall;
  cudaError_t e = launch_prepare();
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(P.zmax, 0x00, nkey * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(P.zmin, 0xff, nkey * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(P.satq, 0, sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  const bool opt = P.opt != 0;
  const size_t s1 = cell_smem_bytes(P.kall, P.mixed != 0, opt);
  const size_t s2 = column_smem_bytes(P.kall, opt);
  dim3 g1((P.gall + CELL_TG - 1) / CELL_TG, P.lall);
  if (ev) cudaEventRecord(ev[0], stream);
  if (opt && P.mixed) nsw6_cell_kernel<FloatMath, float, true><<<g1, CELL_THREADS, s1, stream>>>(P, consts_to_float(C));
  else if (opt) nsw6_cell_kernel<FastMath, double, true><<<g1, CELL_THREADS, s1, stream>>>(P, C);
  else if (P.mixed) nsw6_cell_kernel<FloatMath, float><<<g1, CELL_THREADS, s1, stream>>>(P, consts_to_float(C));
  else if (P.math_lib) nsw6_cell_kernel<LibMath, double><<<g1, CELL_THREADS, s1, stream>>>(P, C);
  else nsw6_cell_kernel<FastMath, double><<<g1, CELL_THREADS, s1, stream>>>(P, C);
  if (ev) cudaEventRecord(ev[1], stream);
  if (before_column && (e = cudaStreamWaitEvent(stream, before_column, 0)) != cudaSuccess) return e;
  const int tg = column_tile(P.kall);
  dim3 g2((P.gall + tg - 1) / tg, P.lall);
  const int nt = column_threads(P.kall);
  // every thread of the column kernel keeps at most 4 (tile 16) or 5 (tile 8) cells
  if ((size_t)nt * (tg == 16 ? 4 : 5) < (size_t)P.kall * tg) return cudaErrorInvalidConfiguration;
  if (tg == 16) {
    if (opt && P.mixed) nsw6_column_kernel<16, FastMath, true, true><<<g2, nt, s2, stream>>>(P, C);
    else if (opt) nsw6_column_kernel<16, FastMath, false, true><<<g2, nt, s2, stream>>>(P, C);
    else if (P.mixed) nsw6_column_kernel<16, FastMath, true><<<g2, nt, s2, stream>>>(P, C);
    else if (P.math_lib) nsw6_column_kernel<16, LibMath, false><<<g2, nt, s2, stream>>>(P, C);
    else nsw6_column_kernel<16, FastMath, false><<<g2, nt, s2, stream>>>(P, C);
  } else {
    if (opt && P.mixed) nsw6_column_kernel<8, FastMath, true, true><<<g2, nt, s2, stream>>>(P, C);
    else if (opt) nsw6_column_kernel<8, FastMath, false, true><<<g2, nt, s2, stream>>>(P, C);
    else if (P.mixed) nsw6_column_kernel<8, FastMath, true><<<g2, nt, s2, stream>>>(P, C);
    else if (P.math_lib) nsw6_column_kernel<8, LibMath, false><<<g2, nt, s2, stream>>>(P, C);
    else nsw6_column_kernel<8, FastMath, false><<<g2, nt, s2, stream>>>(P, C);
  }
  if (opt && P.mixed) nsw6_satadj_kernel<FastMath, true, true><<<SAT_BLOCKS, SAT_THREADS, 0, stream>>>(P, C);
  else if (opt) nsw6_satadj_kernel<FastMath, false, true><<<SAT_BLOCKS, SAT_THREADS, 0, stream>>>(P, C);
  else if (P.mixed) nsw6_satadj_kernel<FastMath, true, false><<<SAT_BLOCKS, SAT_THREADS, 0, stream>>>(P, C);
  else if (P.math_lib) nsw6_satadj_kernel<LibMath, false, false><<<SAT_BLOCKS, SAT_THREADS, 0, stream>>>(P, C);
  else nsw6_satadj_kernel<FastMath, false, false><<<SAT_BLOCKS, SAT_THREADS, 0, stream>>>(P, C);
  if (ev) cudaEventRecord(ev[2], stream);
  return cudaGetLastError();
}

}  // namespace nsw6
