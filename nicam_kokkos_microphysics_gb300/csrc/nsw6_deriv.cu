// Derivative kernels of the NSW6 step: the serial-column FP64 step (the
// forward of the derivative kernels, checked bit for bit against the
// production kernels), the tangent-linear step and the adjoint step.
//
// One thread walks one whole column (nsw6_column_step.cuh).  The region-wide
// bounds of the flux integrals come from the departure-distance extrema of the
// same state, computed beforehand by the production cell kernel on a copy.
#include <cfloat>
#include <cuda_runtime.h>

#include "nsw6_column_step.cuh"

namespace nsw6 {

namespace {

__device__ __forceinline__ void record_error_d(DevStatus* st, int code, int k, int g, int l, int iters) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->k = k;
    st->g = g;
    st->l = l;
    st->iters = iters;
  }
}

// Index helpers for the all-regions layout.
struct Lay {
  int K, G, lall;
  size_t pld;   // row stride of the [2][..] precipitation arrays
  __device__ __forceinline__ size_t f(int l, int k, int g) const { return ((size_t)l * K + k) * G + g; }
  __device__ __forceinline__ size_t t(int l, int n, int k, int g) const {
    return (((size_t)l * NQ + n) * K + k) * G + g;
  }
  __device__ __forceinline__ size_t c(int l, int g) const { return (size_t)l * G + g; }
  __device__ __forceinline__ size_t p(int r, int l, int g) const { return (size_t)r * pld + (size_t)l * G + g; }
};

// Visits every (argument, index, state slot) the step reads.
template <class T, class V>
__device__ __forceinline__ void for_inputs(ColState<T>& s, const Lay& L, int l, int g, const V& v) {
  for (int k = 0; k < L.K; ++k) {
    const size_t i = L.f(l, k, g);
    v(A_rhog, i, s.rhog[k]);
    v(A_rhoge, i, s.rhoge[k]);
    v(A_rhogvx, i, s.rhogvx[k]);
    v(A_rhogvy, i, s.rhogvy[k]);
    v(A_rhogvz, i, s.rhogvz[k]);
    v(A_rhogw, i, s.rhogw[k]);
    v(A_tem, i, s.tem[k]);
    v(A_vx, i, s.vx[k]);
    v(A_vy, i, s.vy[k]);
    v(A_vz, i, s.vz[k]);
    v(A_gsgam2, i, s.gsgam2[k]);
    v(A_gsgam2h, i, s.gsgam2h[k]);
    v(A_gam2, i, s.gam2[k]);
    v(A_gam2h, i, s.gam2h[k]);
    v(A_z, i, s.z[k]);
    for (int n = 0; n < NQ; ++n) {
      const size_t iq = L.t(l, n, k, g);
      v(A_rhogq, iq, s.rhogq[n][k]);
      v(A_q, iq, s.q[n][k]);
    }
  }
  const size_t ic = L.c(l, g);
  v(A_ix, ic, s.ix);
  v(A_iy, ic, s.iy);
  v(A_iz, ic, s.iz);
  v(A_jx, ic, s.jx);
  v(A_jy, ic, s.jy);
  v(A_jz, ic, s.jz);
}

// Visits every (argument, index, value) the step writes; constant outputs are
// passed as T constants.
template <class T, class V>
__device__ __forceinline__ void for_outputs(ColState<T>& s, const Lay& L, int l, int g, const V& v) {
  for (int k = 0; k < L.K; ++k) {
    const size_t i = L.f(l, k, g);
    v(A_rhog, i, s.rhog[k]);
    v(A_rhogvx, i, s.rhogvx[k]);
    v(A_rhogvy, i, s.rhogvy[k]);
    v(A_rhogvz, i, s.rhogvz[k]);
    v(A_rhogw, i, s.rhogw[k]);
    v(A_rhoge, i, s.rhoge[k]);
    v(A_rho, i, s.rho[k]);
    v(A_tem, i, s.tem[k]);
    v(A_pre, i, s.pre[k]);
    v(A_qd, i, s.qd[k]);
    v(A_re_liquid, i, s.re_liquid[k]);
    v(A_re_cld, i, s.re_cld[k]);
    v(A_GPREC, i, s.GPREC[k]);
    T c0 = T(20.0E-6), z0 = T(0.0), z1 = T(0.0);
    v(A_re_solid, i, c0);
    v(A_GDCLW, i, z0);
    v(A_GDCFRC, i, z1);
    for (int n = 0; n < NQ; ++n) {
      const size_t iq = L.t(l, n, k, g);
      v(A_rhogq, iq, s.rhogq[n][k]);
      v(A_q, iq, s.q[n][k]);
    }
  }
  const size_t ic = L.c(l, g);
  v(A_precip, L.p(0, l, g), s.precip0);
  v(A_precip, L.p(1, l, g), s.precip1);
  T z2 = T(0.0), z3 = T(0.0), z4 = T(0.0), z5 = T(0.0);
  v(A_ISO1, L.p(0, l, g), z2);
  v(A_ISO1, L.p(1, l, g), z3);
  v(A_ISO2, L.p(0, l, g), z4);
  v(A_ISO2, L.p(1, l, g), z5);
  v(A_precip_rhoe, ic, s.p_rhoe);
  v(A_precip_lh_heat, ic, s.lh_heat);
  v(A_precip_rhophi, ic, s.p_rhophi);
  v(A_precip_rhokin, ic, s.p_rhokin);
  v(A_rctop, ic, s.rctop);
  v(A_rwtop, ic, s.rwtop);
  v(A_tctop, ic, s.tctop);
}

// Shared-memory set-up common to the derivative kernels: the grid block and
// the fast-math tables.
__device__ __forceinline__ void stage(const Problem& P, double* grid, double* tab) {
  for (int c = threadIdx.x; c < GF_COUNT * P.kall; c += blockDim.x) grid[c] = P.grid[c];
  for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = P.fmtab[c];
  __syncthreads();
}

}  // namespace

// ---- serial-column FP64 step: the derivative kernels' forward, in place
__global__ void __launch_bounds__(AD_THREADS) nsw6_serial_kernel(Problem P, Consts C, ArgPtrs x) {
  __shared__ double grid[GF_COUNT * KA];
  __shared__ double tab[FM_TABLE_DOUBLES];
  stage(P, grid, tab);
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  const Lay L{P.kall, P.gall, P.lall, P.prec_ld};
  const int l = blockIdx.y;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= P.gall) return;
  ColState<double> s;
  ColWork<double> w;
  for_inputs(s, L, l, g, [&](int a, size_t i, double& d) { d = x.a[a][i]; });
  int bmn[6][KA], bmx[6][KA];
  column_bounds(grid + GF_GZH * P.kall, grid + GF_GZSHIFT * P.kall, P.kall, P.kmin, P.kmax,
                P.zmax + (size_t)l * 6 * P.kall, P.zmin + (size_t)l * 6 * P.kall, bmn, bmx);
  int err = 0, ek = 0, eit = 0;
  column_step<double, FastMath>(C, C, fm, fm, grid, P.kall, P.dt, P.rdt, P.hdt2, P.sdt3, P.itelim, bmn, bmx, s, w,
                                &err, &ek, &eit);
  if (err) record_error_d(P.status, err, ek, g, l, eit);
  for_outputs(s, L, l, g, [&](int a, size_t i, double& d) { x.a[a][i] = d; });
}

// ---- tangent-linear step: x <- M(x), dx <- M'(x) dx (+ M_p dp)
__global__ void __launch_bounds__(AD_THREADS) nsw6_tlm_kernel(Problem P, Consts C, ArgPtrs x, ArgPtrs dx,
                                                              const double* params, const double* dparams) {
  __shared__ double grid[GF_COUNT * KA];
  __shared__ double tab[FM_TABLE_DOUBLES];
  stage(P, grid, tab);
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  const ADMath<Dual> mth{fm};
  const Lay L{P.kall, P.gall, P.lall, P.prec_ld};
  const int l = blockIdx.y;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= P.gall) return;
  Dual p[7];
  for (int i = 0; i < 7; ++i) p[i] = Dual(params[i], dparams ? dparams[i] : 0.0);
  ConstsT<Dual> CT;
  consts_with_params(C, p, CT);
  ColState<Dual> s;
  ColWork<Dual> w;
  for_inputs(s, L, l, g, [&](int a, size_t i, Dual& d) { d = Dual(x.a[a][i], dx.a[a][i]); });
  int bmn[6][KA], bmx[6][KA];
  column_bounds(grid + GF_GZH * P.kall, grid + GF_GZSHIFT * P.kall, P.kall, P.kmin, P.kmax,
                P.zmax + (size_t)l * 6 * P.kall, P.zmin + (size_t)l * 6 * P.kall, bmn, bmx);
  int err = 0, ek = 0, eit = 0;
  column_step<Dual, ADMath<Dual>>(CT, C, mth, fm, grid, P.kall, P.dt, P.rdt, P.hdt2, P.sdt3, P.itelim, bmn, bmx, s,
                                  w, &err, &ek, &eit);
  if (err) record_error_d(P.status, err, ek, g, l, eit);
  for_outputs(s, L, l, g, [&](int a, size_t i, Dual& d) {
    x.a[a][i] = d.v;
    dx.a[a][i] = d.d;
  });
}

// ------------------------------------------------------------------ adjoint in stages
// The adjoint step differentiates every part with one thread per cell:
//   1. the cell phase's forward (per cell), its outputs Y: in the recorded
//      form nsw6_adj_cellfwd_kernel below; in the hand-written form (the
//      default) adj_cell_save_kernel (nsw6_adjoint.cu), which also keeps a
//      checkpoint of the costly forward values;
//   2. the column phase's adjoint around Y in level-parallel stages
//      (nsw6_adjoint.cu): adjoints of the step's inputs it reads directly
//      (into xb) and of the cell phase's outputs (YB);
//   3. the adjoint of the cell phase (per cell): adjoints of the cell inputs
//      (into xb) and of the parameters; recorded on a tape by
//      nsw6_adj_cell_kernel below, or swept by hand from the checkpoint by
//      adj_cell_hw_kernel (nsw6_adjoint.cu).
// Y / YB layout: [ADJ_NF][lall][kall][gall], fields below.
enum AdjField {
  Y_RHOG, Y_RHOGE, Y_TEM, Y_RHOGQ, Y_Q = Y_RHOGQ + 6,   // Y_Q + n - 1 for q[n], n = 1..5
  Y_VT = Y_Q + 5,   // fall speeds: Y_VT + 0 Vtr, + 1 Vts, + 2 Vtg, + 3 Vti (0 unless QI sediments)
  Y_RE = Y_VT + 4, Y_RECLD, Y_RCTOP, Y_TCTOP, ADJ_NF
};

// OPT: the cell physics with the scheme switches (the CCN field a constant input).
template <bool OPT>
__global__ void __launch_bounds__(256) nsw6_adj_cellfwd_kernel(Problem P, Consts C, ArgPtrs x, double* Y) {
  __shared__ double tab[FM_TABLE_DOUBLES];
  for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = P.fmtab[c];
  __syncthreads();
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  const Lay L{P.kall, P.gall, P.lall, P.prec_ld};
  const size_t NC = (size_t)P.lall * P.kall * P.gall;
  const int nint = P.kmax - P.kmin + 1;
  const size_t ncell = (size_t)P.lall * nint * P.gall;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    const int g = (int)(c % P.gall);
    const int k = P.kmin + (int)((c / P.gall) % nint);
    const int l = (int)(c / ((size_t)P.gall * nint));
    const size_t i = L.f(l, k, g);
    CellIn in;
    in.rhog = x.a[A_rhog][i];
    in.tem = x.a[A_tem][i];
    in.gsgam2 = x.a[A_gsgam2][i];
    in.q0 = x.a[A_q][L.t(l, 0, k, g)];
    for (int n = 0; n < 6; ++n) in.rhogq[n] = x.a[A_rhogq][L.t(l, n, k, g)];
    in.unccn = (OPT && x.a[A_unccn]) ? x.a[A_unccn][i] : 0.0;
    CellOut o;
    nsw6_cell<FastMath, double, double, OPT>(C, fm, P.dt, P.rdt, in, o);
    Y[Y_RHOG * NC + i] = o.rhog;
    Y[Y_RHOGE * NC + i] = o.rhoge;
    Y[Y_TEM * NC + i] = o.tem;
    for (int n = 0; n < 6; ++n) Y[(Y_RHOGQ + n) * NC + i] = o.rhogq[n];
    for (int n = 1; n < 6; ++n) Y[(Y_Q + n - 1) * NC + i] = o.q[n];
    Y[(Y_VT + 0) * NC + i] = o.Vtr;
    Y[(Y_VT + 1) * NC + i] = o.Vts;
    Y[(Y_VT + 2) * NC + i] = o.Vtg;
    Y[(Y_VT + 3) * NC + i] = o.Vti;
    Y[Y_RE * NC + i] = o.rceff;
    Y[Y_RECLD * NC + i] = o.rceff_cld;
    Y[Y_RCTOP * NC + i] = o.rctop;
    Y[Y_TCTOP * NC + i] = o.tctop;
  }
}

__device__ __forceinline__ void tape_bind(const TapeMem& tm) {
  Tape& t = tape();
  t.pa = tm.pa;
  t.pb = tm.pb;
  t.da = tm.da;
  t.db = tm.db;
  t.adj = tm.adj;
  t.nslot = tm.nslot;
  t.slot = blockIdx.x * blockDim.x + threadIdx.x;
  t.cap = tm.cap;
  t.count_only = tm.count_only;
}

// done[cell] (may be null): set once a cell's adjoint has been added; cells
// already done are skipped, so that a launch repeated with a longer tape after
// an overflow adds each cell once.
template <bool OPT>
__global__ void __launch_bounds__(AD_THREADS, 3) nsw6_adj_cell_kernel(Problem P, Consts C, ArgPtrs x, ArgPtrs xb,
                                                                   const double* YB, TapeMem tm,
                                                                   const double* params, double* pbar,
                                                                   int* tape_max, int* done) {
  __shared__ double tab[FM_TABLE_DOUBLES];
  __shared__ double red[7][AD_THREADS];
  for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = P.fmtab[c];
  __syncthreads();
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  const ADMath<RVar> mth{fm};
  const Lay L{P.kall, P.gall, P.lall, P.prec_ld};
  const size_t NC = (size_t)P.lall * P.kall * P.gall;
  const int nint = P.kmax - P.kmin + 1;
  const long long ncell = (long long)P.lall * nint * P.gall;
  tape_bind(tm);
  Tape& t = tape();
  double pacc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (long long c = t.slot; c < ncell; c += t.nslot) {
    if (done && done[c]) continue;
    const int g = (int)(c % P.gall);
    const int k = P.kmin + (int)((c / P.gall) % nint);
    const int l = (int)(c / ((long long)P.gall * nint));
    const size_t i = L.f(l, k, g);
    t.n = 0;
    t.overflow = 0;
    RVar p[7];
    for (int j = 0; j < 7; ++j) p[j] = leaf(params[j]);
    ConstsT<RVar> CT;
    consts_with_params(C, p, CT);
    CellInT<RVar> in;
    in.rhog = leaf(x.a[A_rhog][i]);
    in.tem = leaf(x.a[A_tem][i]);
    in.gsgam2 = leaf(x.a[A_gsgam2][i]);
    in.q0 = leaf(x.a[A_q][L.t(l, 0, k, g)]);
    for (int n = 0; n < 6; ++n) in.rhogq[n] = leaf(x.a[A_rhogq][L.t(l, n, k, g)]);
    in.unccn = RVar((OPT && x.a[A_unccn]) ? x.a[A_unccn][i] : 0.0);
    CellOutT<RVar> o;
    nsw6_cell<ADMath<RVar>, RVar, RVar, OPT>(CT, mth, P.dt, P.rdt, in, o);
    atomicMax(tape_max, t.overflow ? t.cap + 1 : t.n);
    if (t.overflow || t.count_only) continue;
    for (int e = 0; e < t.n; ++e) t.adj[(size_t)e * t.nslot + t.slot] = 0.0;
    auto seed = [&](const RVar& d, int f) {
      if (d.id >= 0) adj_of(d) += YB[f * NC + i];
    };
    seed(o.rhog, Y_RHOG);
    seed(o.rhoge, Y_RHOGE);
    seed(o.tem, Y_TEM);
    for (int n = 0; n < 6; ++n) seed(o.rhogq[n], Y_RHOGQ + n);
    for (int n = 1; n < 6; ++n) seed(o.q[n], Y_Q + n - 1);
    seed(o.Vtr, Y_VT + 0);
    seed(o.Vts, Y_VT + 1);
    seed(o.Vtg, Y_VT + 2);
    seed(o.Vti, Y_VT + 3);
    seed(o.rceff, Y_RE);
    seed(o.rceff_cld, Y_RECLD);
    if (k == P.kmax) {
      seed(o.rctop, Y_RCTOP);
      seed(o.tctop, Y_TCTOP);
    }
    tape_reverse();
    auto add = [&](const RVar& d, int a, size_t idx) {
      if (d.id >= 0) xb.a[a][idx] += adj_of(d);
    };
    add(in.rhog, A_rhog, i);
    add(in.tem, A_tem, i);
    add(in.gsgam2, A_gsgam2, i);
    add(in.q0, A_q, L.t(l, 0, k, g));
    for (int n = 0; n < 6; ++n) add(in.rhogq[n], A_rhogq, L.t(l, n, k, g));
    for (int j = 0; j < 7; ++j) pacc[j] += adj_of(p[j]);
    if (done) done[c] = 1;
  }
  for (int j = 0; j < 7; ++j) red[j][threadIdx.x] = pacc[j];
  __syncthreads();
  if (threadIdx.x < 7) {
    double sum = 0.0;
    for (int j = 0; j < (int)blockDim.x; ++j) sum += red[threadIdx.x][j];
    atomicAdd(&pbar[threadIdx.x], sum);
  }
}

// ------------------------------------------------------------------ launchers
cudaError_t launch_serial(const Problem& P, const Consts& C, const ArgPtrs& x, cudaStream_t stream) {
  dim3 grid((P.gall + AD_THREADS - 1) / AD_THREADS, P.lall);
  nsw6_serial_kernel<<<grid, AD_THREADS, 0, stream>>>(P, C, x);
  return cudaGetLastError();
}

cudaError_t launch_tlm(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& dx, const double* params,
                       const double* dparams, cudaStream_t stream) {
  dim3 grid((P.gall + AD_THREADS - 1) / AD_THREADS, P.lall);
  nsw6_tlm_kernel<<<grid, AD_THREADS, 0, stream>>>(P, C, x, dx, params, dparams);
  return cudaGetLastError();
}

constexpr int ADJ_NFIELDS = ADJ_NF;

cudaError_t launch_adj_cellfwd(const Problem& P, const Consts& C, const ArgPtrs& x, double* Y, cudaStream_t stream) {
  if (P.opt)
    nsw6_adj_cellfwd_kernel<true><<<152 * 4, 256, 0, stream>>>(P, C, x, Y);
  else
    nsw6_adj_cellfwd_kernel<false><<<152 * 4, 256, 0, stream>>>(P, C, x, Y);
  return cudaGetLastError();
}

cudaError_t launch_adj_cell(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& xb, const double* YB,
                            const TapeMem& tm, const double* params, double* pbar, int* tape_max, int* done,
                            cudaStream_t stream) {
  if (P.opt)
    nsw6_adj_cell_kernel<true><<<tm.nslot / AD_THREADS, AD_THREADS, 0, stream>>>(P, C, x, xb, YB, tm, params, pbar,
                                                                         tape_max, done);
  else
    nsw6_adj_cell_kernel<false><<<tm.nslot / AD_THREADS, AD_THREADS, 0, stream>>>(P, C, x, xb, YB, tm, params, pbar,
                                                                         tape_max, done);
  return cudaGetLastError();
}

int adj_nfields() { return ADJ_NFIELDS; }

}  // namespace nsw6
