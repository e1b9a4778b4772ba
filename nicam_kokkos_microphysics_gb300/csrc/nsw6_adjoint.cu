// Level-parallel adjoint of the column phase of the NSW6 step.
//
// The column phase (everything after the per-cell physics: departure
// distances, the transport of QR, (QI,) QS, QG, KIN2EIN, thermodynamics, the
// saturation adjustment and the closing negative filter) is split at the
// points where a value computed at one level is read at another, into four
// per-cell stages:
//
//   S1  departure distances (vadv1d_prep, mod_vadv1d.cpp:231-391) from the
//       fall speeds, the kinetic energies and the eight flux sources of each
//       sedimenting tracer (mod_precip_transport.cpp:767-900) of one cell;
//   S2  one flux integral of vadv1d_getflux_new (mod_vadv1d.cpp:393-450) of
//       one cell (a work item per cell and flux);
//   S3  the flux divergences, surface fluxes and the application of the
//       tendencies (mod_precip_transport.cpp:782-989) of one cell;
//   S4  KIN2EIN (:991-1011), the final thermodynamic state, the saturation
//       adjustment (mod_satadjust.cpp:274-362, 771-896) and the negative filter
//       of one cell.
//
// Each stage is a function of one cell written over the scalar type T, its
// inputs read through an accessor.  The forward kernels (T = double) store the
// stage outputs.  The adjoint kernels (adj_s*_hw_kernel) recompute one cell's
// stage and sweep it back statement by statement, adding the adjoints of its
// inputs wherever they live (another level, the cell phase's outputs, the
// caller's arrays): with atomics where other threads add to the same place,
// in place where only the thread does (S3 in gather form, each cell
// collecting the adjoints of the fluxes it feeds).  Adjoint mode 1 runs the
// recorded form instead (T = RVar: the stage re-recorded on a short per-thread
// tape, seeded, swept), which checks the hand-written sweeps.  Every cell of
// every column runs in parallel.  This file also holds the cell phase's
// hand-written adjoint kernels (its forward with a checkpoint of the costly
// values, then the reverse sweep from it; nsw6_cell_adjoint.cuh).
//
// The arithmetic is that of the serial column step (nsw6_column_step.cuh),
// which reproduces the production kernels bit for bit; discrete choices
// (departure cells, flux bounds, the small-flux filter, limiter branches) are
// held at the forward's values and the Newton temperature is differentiated
// implicitly, as there.
#include <cfloat>
#include <cuda_runtime.h>

#include "nsw6_cell_adjoint.cuh"
#include "nsw6_column_step.cuh"

namespace nsw6 {

// Cell-phase output fields (Y / YB layout of nsw6_deriv.cu).  Fall speeds:
// YS_VT + 0 Vtr, + 1 Vts, + 2 Vtg, + 3 Vti (0 unless QI sediments).
enum AdjFieldS {
  YS_RHOG, YS_RHOGE, YS_TEM, YS_RHOGQ, YS_Q = YS_RHOGQ + 6, YS_VT = YS_Q + 5, YS_RE = YS_VT + 4, YS_RECLD,
  YS_RCTOP, YS_TCTOP, ADJ_Y_FIELDS
};

// Sedimenting tracer t of ntr in the transport's order (mod_mp_nsw6.cpp:596-599,
// mod_precip_transport.cpp:767): QR, QS, QG, or QR, QI, QS, QG when QI
// sediments ("4WATER"); nq its tracer index, vt its fall speed's Y field.
struct SedTracer {
  int nq, vt;
};
__device__ __forceinline__ SedTracer sed_tracer(int t, int ntr) {
  if (t == 0) return {I_QR, YS_VT + 0};
  if (ntr == 4 && t == 1) return {I_QI, YS_VT + 3};
  const int u = ntr == 4 ? t - 1 : t;   // 1: QS, 2: QG
  return {u == 1 ? I_QS : I_QG, YS_VT + u};
}
constexpr int MAX_TR = 4;

// Work fields of the staged column adjoint: [NWF][lall][kall][gall], laid out
// for up to four sedimenting tracers (t < ntr are used).
enum WorkField {
  W_ZDIS = 0,                  // 2 ntr departure distances: row t full, row ntr + t half
  W_KINH = 2 * MAX_TR, W_KINV, // kinetic energies of the transport's input state
  W_RHOF,                      // flux sources, tracer t, flux j: W_RHOF + 8 t + j (j < 6 full, 6..7 half)
  W_F = W_RHOF + 8 * MAX_TR,   // fluxes, same order
  W_RHOG_N = W_F + 8 * MAX_TR, W_RHOGE_N, W_RVX_N, W_RVY_N, W_RVZ_N, W_RW_N,
  W_RQ_N,                      // 6 tracers
  W_KINH_N = W_RQ_N + 6, W_KINV_N,
  NWF
};

// Seeds (output adjoints) of the column phase, copied from the caller's
// adjoint arrays before any input adjoint is added there: [NSF][lall][kall][gall]
// then the six column outputs [6][lall][gall].
enum SeedField {
  SF_RHOG, SF_RHOGE, SF_RVX, SF_RVY, SF_RVZ, SF_RW, SF_RHO, SF_TEM, SF_PRE, SF_QD, SF_GPREC,
  SF_RQ, SF_Q = SF_RQ + 6, NSF = SF_Q + 6
};
enum SeedColumn { SC_PRECIP0, SC_PRECIP1, SC_LH, SC_RHOE, SC_RHOPHI, SC_RHOKIN, NSC };

constexpr int STAGE_THREADS = AD_THREADS;
constexpr int MAX_LEAVES = 96;
constexpr int ERR_ADJ_CAPACITY = 5;   // a tape or the leaf log of a stage overflowed (NSW6_ERR_UNSUPPORTED)

namespace {

struct LayS {
  int K, G, lall;
  size_t pld;   // row stride of the [2][..] precipitation arrays
  FastDiv dG, dK;   // by G and by K: the cell index splits on 32 bits (lall kall gall < 2^32, nsw6_create)
  // c = (l K + k) G + g -> l, k, g
  __device__ __forceinline__ void split(size_t c, int& l, int& k, int& g) const {
    const unsigned ci = (unsigned)c, q = dG.div(ci), q2 = dK.div(q);
    g = (int)(ci - q * (unsigned)G);
    k = (int)(q - q2 * (unsigned)K);
    l = (int)q2;
  }
  __device__ __forceinline__ size_t f(int l, int k, int g) const { return ((size_t)l * K + k) * G + g; }
  __device__ __forceinline__ size_t t(int l, int n, int k, int g) const {
    return (((size_t)l * NQ + n) * K + k) * G + g;
  }
  __device__ __forceinline__ size_t c(int l, int g) const { return (size_t)l * G + g; }
  __device__ __forceinline__ size_t p(int r, int l, int g) const { return (size_t)r * pld + (size_t)l * G + g; }
};

__device__ __forceinline__ void record_err(DevStatus* st, int code, int k, int g, int l, int iters) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->k = k;
    st->g = g;
    st->l = l;
    st->iters = iters;
  }
}

// Everything a stage reads, and where the adjoints of what it reads go.
struct StageIO {
  Problem P;
  LayS L;
  size_t NC;
  ArgPtrs x, xb;
  const double* Y;
  double* YB;
  double* W;
  double* WB;
  const double* SB;     // seeds [NSF][NC] then [NSC][lall][gall]
  const int* bnd;       // flux bounds [lall][2][2 MAX_TR][kall]: bmn then bmx, rows as W_ZDIS
  int kin2kin;          // the KIN2KIN switch: S4, not S3, gives the final momenta
};

// Where a leaf's adjoint is added.
enum LeafKind { LK_W = 0, LK_Y = 1, LK_X = 2 };

struct LeafLog {
  int n, overflow;
  int code[MAX_LEAVES];
  int id[MAX_LEAVES];
  size_t idx[MAX_LEAVES];
};

// Input accessor.  T = double: the stored values.  T = RVar: a new leaf per
// read, logged with the place its adjoint belongs to.
template <class T>
struct In;

template <>
struct In<double> {
  const StageIO& io;
  int l, g;
  __device__ double w(int f, int kk) const { return io.W[f * io.NC + io.L.f(l, kk, g)]; }
  __device__ double y(int f, int kk) const { return io.Y[f * io.NC + io.L.f(l, kk, g)]; }
  __device__ double x(int a, size_t i) const { return io.x.a[a][i]; }
};

template <>
struct In<RVar> {
  const StageIO& io;
  int l, g;
  LeafLog* log;
  __device__ RVar put(int kind, int f, size_t i, double v) const {
    const RVar r = leaf(v);
    if (r.id < 0) return r;   // tape full: the stage reports the overflow
    if (log->n >= MAX_LEAVES) {
      log->overflow = 1;
      return r;
    }
    log->code[log->n] = kind * 4096 + f;
    log->id[log->n] = r.id;
    log->idx[log->n] = i;
    ++log->n;
    return r;
  }
  __device__ RVar w(int f, int kk) const {
    const size_t i = io.L.f(l, kk, g);
    return put(LK_W, f, i, io.W[f * io.NC + i]);
  }
  __device__ RVar y(int f, int kk) const {
    const size_t i = io.L.f(l, kk, g);
    return put(LK_Y, f, i, io.Y[f * io.NC + i]);
  }
  __device__ RVar x(int a, size_t i) const { return put(LK_X, a, i, io.x.a[a][i]); }
};

// State fields the column phase reads: the cell phase's output at interior
// levels, the caller's array at the halo levels.
template <class T>
__device__ __forceinline__ T st_rhog(const In<T>& in, int kk) {
  return (kk >= in.io.P.kmin && kk <= in.io.P.kmax) ? in.y(YS_RHOG, kk) : in.x(A_rhog, in.io.L.f(in.l, kk, in.g));
}
template <class T>
__device__ __forceinline__ T st_rhoge(const In<T>& in, int kk) {
  return (kk >= in.io.P.kmin && kk <= in.io.P.kmax) ? in.y(YS_RHOGE, kk) : in.x(A_rhoge, in.io.L.f(in.l, kk, in.g));
}
template <class T>
__device__ __forceinline__ T st_tem(const In<T>& in, int kk) {
  return (kk >= in.io.P.kmin && kk <= in.io.P.kmax) ? in.y(YS_TEM, kk) : in.x(A_tem, in.io.L.f(in.l, kk, in.g));
}
template <class T>
__device__ __forceinline__ T st_rhogq(const In<T>& in, int n, int kk) {
  return (kk >= in.io.P.kmin && kk <= in.io.P.kmax) ? in.y(YS_RHOGQ + n, kk)
                                                      : in.x(A_rhogq, in.io.L.t(in.l, n, kk, in.g));
}
template <class T>
__device__ __forceinline__ T st_q(const In<T>& in, int n, int kk) {   // n >= 1
  return (kk >= in.io.P.kmin && kk <= in.io.P.kmax) ? in.y(YS_Q + n - 1, kk)
                                                      : in.x(A_q, in.io.L.t(in.l, n, kk, in.g));
}
template <class T>
__device__ __forceinline__ T xf(const In<T>& in, int a, int kk) {
  return in.x(a, in.io.L.f(in.l, kk, in.g));
}
template <class T>
__device__ __forceinline__ T xc(const In<T>& in, int a) {
  return in.x(a, in.io.L.c(in.l, in.g));
}

// ------------------------------------------------------------------ stages
// S1: departure distances, kinetic energies and flux sources of cell (l, k, g).
// MIX (T = double): the departure distances of the mixed-precision step, in
// FP32 from the FP32 reciprocal rows grf (rdgz, rdgzh, rdzs, rdzsh) as its
// cell kernel forms them, so that the flux bounds and departure cells are the
// mixed step's.
template <class T, bool MIX = false, class O>
__device__ void stage1(const In<T>& in, const double* gr, int k, const O& out, const float* grf = nullptr) {
  const Problem& P = in.io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const double* rdgz = gr + GF_RDGZ * K;
  const double* rdgzh = gr + GF_RDGZH * K;
  const double* rdzs = gr + GF_RDZS * K;
  const double* rdzsh = gr + GF_RDZSH * K;
  const double* afact = gr + GF_AFACT * K;
  const double* bfact = gr + GF_BFACT * K;
  const bool interior = (k >= kmin && k <= kmax);
  const int ntr = P.ntr;
  // fall speeds at levels k-3 .. k+1 (zero outside the interior)
  T vt[MAX_TR][5];
  for (int t = 0; t < ntr; ++t)
    for (int j = 0; j < 5; ++j) {
      const int kk = k - 3 + j;
      vt[t][j] = (interior && kk >= kmin && kk <= kmax) ? in.y(sed_tracer(t, ntr).vt, kk) : T(0.0);
    }
  float vtf[MIX ? MAX_TR : 1][5];
  if constexpr (MIX)
    for (int t = 0; t < ntr; ++t)
      for (int j = 0; j < 5; ++j) vtf[t][j] = float(vt[t][j]);
  for (int r = 0; r < 2 * ntr; ++r) {
    const int t = r % ntr, half = r / ntr;
    const int mkmin = half ? kmin + 1 : kmin;
    T z = T(0.0);
    if constexpr (MIX) {
      if (k >= mkmin && k <= kmax) {
        auto col = [&](int j) { return vtf[t][j - k + 3]; };
        const float dtf = float(P.dt), hdt2f = float(P.hdt2), sdt3f = float(P.sdt3);
        float zf;
        if (!half) {
          auto wp = [&](int j) { return col(j); };
          zf = vadv_zdis<float>(wp, grf, grf + 2 * K, k, mkmin, kmax, dtf, hdt2f, sdt3f);
        } else {
          auto wp = [&](int j) { return (j >= kmin + 1 && j <= kmax - 1) ? 0.5f * (col(j) + col(j - 1)) : 0.0f; };
          zf = vadv_zdis<float>(wp, grf + K, grf + 3 * K, k, mkmin, kmax, dtf, hdt2f, sdt3f);
        }
        z = T(double(zf));
      }
      out(W_ZDIS + r, z);
      continue;
    }
    if (k >= mkmin && k <= kmax) {
      auto col = [&](int j) { return vt[t][j - k + 3]; };
      if (!half) {
        auto wp = [&](int j) { return col(j); };
        z = vadv_zdis<T>(wp, rdgz, rdzs, k, mkmin, kmax, T(P.dt), T(P.hdt2), T(P.sdt3));
      } else {
        auto wp = [&](int j) { return (j >= kmin + 1 && j <= kmax - 1) ? T(0.5) * (col(j) + col(j - 1)) : T(0.0); };
        z = vadv_zdis<T>(wp, rdgzh, rdzsh, k, mkmin, kmax, T(P.dt), T(P.hdt2), T(P.sdt3));
      }
    }
    out(W_ZDIS + r, z);
  }
  // metric factors and kinetic energy (mod_precip_transport.cpp:715-770)
  T rgs = T(0.0), kinh = T(0.0), kinv = T(0.0);
  if (interior) rgs = xf(in, A_gam2, k) / xf(in, A_gsgam2, k);
  const T vx = xf(in, A_vx, k), vy = xf(in, A_vy, k), vz = xf(in, A_vz, k);
  const T vi = vx * xc(in, A_ix) + vy * xc(in, A_iy) + vz * xc(in, A_iz);
  const T vj = vx * xc(in, A_jx) + vy * xc(in, A_jy) + vz * xc(in, A_jz);
  if (interior) {
    const T rvx = xf(in, A_rhogvx, k), rvy = xf(in, A_rhogvy, k), rvz = xf(in, A_rhogvz, k);
    kinh = 0.5 * (rvx * rvx + rvy * rvy + rvz * rvz) / st_rhog(in, k);
  }
  const bool hk = (k >= kmin + 1 && k <= kmax);
  T rw = T(0.0);
  if (hk) {
    const T gh = xf(in, A_gsgam2h, k);
    const T c2w0 = afact[k] / xf(in, A_gsgam2, k) * gh;
    const T c2w1 = bfact[k] / xf(in, A_gsgam2, k - 1) * gh;
    rw = xf(in, A_rhogw, k);
    kinv = 0.5 * (rw * rw) / (c2w0 * st_rhog(in, k) + c2w1 * st_rhog(in, k - 1));
  }
  out(W_KINH, kinh);
  out(W_KINV, kinv);
  // flux sources of the sedimenting tracers (mod_precip_transport.cpp:776-808, 864-882)
  const T tem = interior ? st_tem(in, k) : T(0.0);
  const T zz = interior ? xf(in, A_z, k) : T(0.0);
  T rgsh = T(0.0);
  if (hk) rgsh = xf(in, A_gam2h, k) / xf(in, A_gsgam2h, k);
  for (int t = 0; t < ntr; ++t) {
    const int nq = sed_tracer(t, ntr).nq;
    T base = T(0.0), qn = T(0.0);
    if (interior) {
      base = st_rhogq(in, nq, k) * rgs;
      qn = st_q(in, nq, k);
    }
    out(W_RHOF + 8 * t + 0, base);
    out(W_RHOF + 8 * t + 1, base * CVDRY * tem);
    out(W_RHOF + 8 * t + 2, base * GRAV * zz);
    out(W_RHOF + 8 * t + 3, qn * rgs * kinh);
    out(W_RHOF + 8 * t + 4, base * vi);
    out(W_RHOF + 8 * t + 5, base * vj);
    T qh = T(0.0), h1 = T(0.0);
    if (hk) {
      qh = 0.5 * (qn + st_q(in, nq, k - 1)) * rgsh;
      h1 = qh * rw;
    }
    out(W_RHOF + 8 * t + 6, qh * kinv);
    out(W_RHOF + 8 * t + 7, h1);
  }
}

// S2: flux j (tracer j / 8, source j % 8) of cell (l, k, g).
template <class T>
__device__ T stage2(const In<T>& in, const double* gr, int k, int j) {
  const Problem& P = in.io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const int t = j / 8, f = j % 8;
  const bool full = f < 6;
  const int mkmin = full ? kmin : kmin + 1;
  if (k < mkmin || k > kmax) return T(0.0);
  const int r = full ? t : P.ntr + t;
  const int* bmn = in.io.bnd + ((size_t)in.l * 2 + 0) * 2 * MAX_TR * K;
  const int* bmx = in.io.bnd + ((size_t)in.l * 2 + 1) * 2 * MAX_TR * K;
  // the integral's range: the half levels use the full-level kcell_max
  // (mod_precip_transport.cpp:890, 892)
  const int lo = bmn[r * K + k];
  const int hi = bmx[t * K + k];
  const double* zh = gr + (full ? GF_GZH : GF_GZSHIFT) * K;
  const double* dz = gr + (full ? GF_DGZ : GF_DGZH) * K;
  const double zv = in.io.W[(W_ZDIS + r) * in.io.NC + in.io.L.f(in.l, k, in.g)];
  const int kc = departure_cell_t(zh, k, zv, lo, bmx[r * K + k], mkmin, kmax);
  const int src = W_RHOF + 8 * t + f;
  T acc = T(0.0);
  T zdis = in.w(W_ZDIS + r, k);
  if (!(lo == k && hi == k)) {
    for (int k2 = lo; k2 <= hi; ++k2)
      acc = fmaR(in.w(src, k2), T(k2 > kc ? dz[k2] : (k2 < kc ? -dz[k2] : 0.0)), acc);
    if (hi != kc) zdis = zdis - T(hi > kc ? dz[hi] : -dz[hi]);
  }
  acc = fmaR(in.w(src, kc), zdis, acc);
  return fabsR(acc) >= T(EPS) ? acc : T(0.0);
}

// S3: divergences, surface fluxes and the updated state of cell (l, k, g).
// o(field, value) for the work fields; fin(seed field, value) for the caller's
// outputs written here (rhogvx/y/z, rhogw, GPREC); col(seed column, value) for
// the surface outputs (k = kmin).
template <class T, class O, class F, class Cc>
__device__ void stage3(const In<T>& in, const double* gr, int k, const O& o, const F& fin, const Cc& col) {
  const Problem& P = in.io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const double* rdgz = gr + GF_RDGZ * K;
  const double* rdgzh = gr + GF_RDGZH * K;
  const double dt = P.dt;
  const bool interior = (k >= kmin && k <= kmax);
  const bool hk = (k >= kmin + 1 && k <= kmax);
  const int ntr = P.ntr;
  T dq[MAX_TR] = {T(0.0), T(0.0), T(0.0), T(0.0)};
  T drhoe = T(0.0), drhophi = T(0.0), dkinh = T(0.0), dkinv = T(0.0), du = T(0.0), dv = T(0.0), dw = T(0.0);
  T acc[6] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
  for (int t = 0; t < ntr; ++t) {
    const int nq = sed_tracer(t, ntr).nq;
    if (interior) {
      for (int f = 0; f < 6; ++f) {
        const T fk = in.w(W_F + 8 * t + f, k), fk1 = in.w(W_F + 8 * t + f, k + 1);
        const T d = (fk1 - fk) * rdgz[k];
        switch (f) {
          case 0:
            dq[t] = -d;
            if (nq == I_QR) fin(SF_GPREC, 0.0 + (-fk / dt));
            break;
          case 1: drhoe = drhoe - d; break;
          case 2: drhophi = drhophi - d; break;
          case 3: dkinh = dkinh - d; break;
          case 4: du = du - d; break;
          default: dv = dv - d; break;
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
    if (hk) {
      for (int w = 0; w < 2; ++w) {
        const T d = (in.w(W_F + 8 * t + 6 + w, k) - in.w(W_F + 8 * t + 6 + w, k - 1)) * rdgzh[k];
        if (w == 0) dkinv = dkinv - d;
        else dw = dw - d;
      }
    }
  }
  if (k == kmin) {
    col(SC_PRECIP0, 0.0 + acc[0]);
    col(SC_PRECIP1, 0.0 + acc[1]);
    col(SC_LH, 0.0 + acc[2]);
    col(SC_RHOE, 0.0 + acc[3]);
    col(SC_RHOPHI, 0.0 + acc[4]);
    col(SC_RHOKIN, 0.0 + acc[5]);
  }
  // apply the tendencies (mod_precip_transport.cpp:956-989)
  T rhoge = st_rhoge(in, k) + drhoe + drhophi;
  o(W_KINH_N, in.w(W_KINH, k) + dkinh);
  o(W_KINV_N, in.w(W_KINV, k) + dkinv);
  const T ix = xc(in, A_ix), iy = xc(in, A_iy), iz = xc(in, A_iz);
  const T jx = xc(in, A_jx), jy = xc(in, A_jy), jz = xc(in, A_jz);
  const T rvx = xf(in, A_rhogvx, k) + du * ix + dv * jx;
  const T rvy = xf(in, A_rhogvy, k) + du * iy + dv * jy;
  const T rvz = xf(in, A_rhogvz, k) + du * iz + dv * jz;
  const T rw = xf(in, A_rhogw, k) + dw;
  o(W_RVX_N, rvx);
  o(W_RVY_N, rvy);
  o(W_RVZ_N, rvz);
  o(W_RW_N, rw);
  fin(SF_RVX, rvx);
  fin(SF_RVY, rvy);
  fin(SF_RVZ, rvz);
  fin(SF_RW, rw);
  T rhog = st_rhog(in, k);
  const T zz = xf(in, A_z, k);
  o(W_RQ_N + I_QV, st_rhogq(in, I_QV, k) + 0.0);
  o(W_RQ_N + I_QC, st_rhogq(in, I_QC, k) + 0.0);
  o(W_RQ_N + I_QR, st_rhogq(in, I_QR, k) + dq[0]);
  rhog = rhog + dq[0];
  rhoge = rhoge - dq[0] * GRAV * zz;
  // (tracers in order QV..QG; QI adds an exact zero unless it sediments)
  const int ts = ntr - 2, tg = ntr - 1;   // QS, QG
  if (ntr == 4) {
    o(W_RQ_N + I_QI, st_rhogq(in, I_QI, k) + dq[1]);
    rhog = rhog + dq[1];
    rhoge = rhoge - dq[1] * GRAV * zz;
  } else {
    o(W_RQ_N + I_QI, st_rhogq(in, I_QI, k) + 0.0);
  }
  o(W_RQ_N + I_QS, st_rhogq(in, I_QS, k) + dq[ts]);
  rhog = rhog + dq[ts];
  rhoge = rhoge - dq[ts] * GRAV * zz;
  o(W_RQ_N + I_QG, st_rhogq(in, I_QG, k) + dq[tg]);
  rhog = rhog + dq[tg];
  rhoge = rhoge - dq[tg] * GRAV * zz;
  o(W_RHOG_N, rhog);
  o(W_RHOGE_N, rhoge);
}

// Vertical kinetic energy of the updated state at half level j.
template <class T>
__device__ __forceinline__ T kinv_new(const In<T>& in, const double* gr, int j) {
  const Problem& P = in.io.P;
  const int K = P.kall;
  if (!(j >= P.kmin + 1 && j <= P.kmax)) return T(0.0);
  const double* afact = gr + GF_AFACT * K;
  const double* bfact = gr + GF_BFACT * K;
  const T gh = xf(in, A_gsgam2h, j);
  const T c2w0 = afact[j] / xf(in, A_gsgam2, j) * gh;
  const T c2w1 = bfact[j] / xf(in, A_gsgam2, j - 1) * gh;
  const T rw = in.w(W_RW_N, j);
  return 0.5 * (rw * rw) / (c2w0 * in.w(W_RHOG_N, j) + c2w1 * in.w(W_RHOG_N, j - 1));
}

// S4: KIN2EIN, thermodynamics, saturation adjustment and negative filter of
// cell (l, k, g); fin(seed field, value) for each output.  Returns the Newton
// status (0, or 3 / 4 with *iters).
template <class T, class F>
__device__ int stage4(const In<T>& in, const Consts& C, const double* gr, const FastMath& fm, int k, const F& fin,
                      int* iters) {
  const Problem& P = in.io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const double* cfact = gr + GF_CFACT * K;
  const double* dfact = gr + GF_DFACT * K;
  const bool interior = (k >= kmin && k <= kmax);
  const bool kin2kin = P.opt && C.opt_kin2kin != 0.0;
  const T rhog = in.w(W_RHOG_N, k);
  const T rrhog = 1.0 / rhog;
  T rhoge = in.w(W_RHOGE_N, k);
  const T gsg = xf(in, A_gsgam2, k);
  if (kin2kin) {
    // KIN2KIN (mod_precip_transport.cpp:1012-1068) in place of KIN2EIN: the
    // transported momenta rescaled to carry the transported kinetic energy,
    // horizontal on [kmin, kmax], vertical on [kmin, kmax + 1]; the other
    // levels pass through
    T rvx = in.w(W_RVX_N, k), rvy = in.w(W_RVY_N, k), rvz = in.w(W_RVZ_N, k), rw = in.w(W_RW_N, k);
    if (k >= kmin && k <= kmax + 1) {
      if (k <= kmax) {
        const T kin_h0 = in.w(W_KINH_N, k) / rhog;
        T vx_t = rvx / rhog, vy_t = rvy / rhog, vz_t = rvz / rhog;
        const T kin_h = 0.5 * (vx_t * vx_t + vy_t * vy_t + vz_t * vz_t);
        if (val_of(kin_h) > 1.0E-20) {
          const T r = sqrtR(fabsR(kin_h0 / kin_h));
          vx_t = vx_t * r;
          vy_t = vy_t * r;
          vz_t = vz_t * r;
        }
        rvx = vx_t * rhog;
        rvy = vy_t * rhog;
        rvz = vz_t * rhog;
      }
      const double* afact = gr + GF_AFACT * K;
      const double* bfact = gr + GF_BFACT * K;
      const T gh = xf(in, A_gsgam2h, k);
      const T c2w0 = afact[k] / gsg * gh;
      const T c2w1 = bfact[k] / xf(in, A_gsgam2, k - 1) * gh;
      const T rhogh = c2w0 * rhog + c2w1 * in.w(W_RHOG_N, k - 1);
      const T kin_v0 = in.w(W_KINV_N, k) / rhogh;
      T w_t = rw / rhogh;
      const T kin_v = 0.5 * (w_t * w_t);
      if (val_of(kin_v) > 1.0E-20) w_t = w_t * sqrtR(fabsR(kin_v0 / kin_v));
      rw = w_t * rhogh;
    }
    fin(SF_RVX, rvx);
    fin(SF_RVY, rvy);
    fin(SF_RVZ, rvz);
    fin(SF_RW, rw);
  } else if (interior) {
    // KIN2EIN (mod_precip_transport.cpp:991-1011): the transported kinetic
    // energy tmp2 less that of the updated state
    const T gh = xf(in, A_gsgam2h, k + 1), rgh = 1.0 / gh;
    const T w2c0 = div_rn(cfact[k] * gsg, gh, rgh);
    const T w2c1 = div_rn(dfact[k] * gsg, gh, rgh);
    const T tmp2 = in.w(W_KINH_N, k) + (w2c0 * in.w(W_KINV_N, k + 1) + w2c1 * in.w(W_KINV_N, k));
    const T rvx = in.w(W_RVX_N, k), rvy = in.w(W_RVY_N, k), rvz = in.w(W_RVZ_N, k);
    const T tmp_h = div_rn(0.5 * (rvx * rvx + rvy * rvy + rvz * rvz), rhog, rrhog);
    const T tmp = tmp_h + (w2c0 * kinv_new(in, gr, k + 1) + w2c1 * kinv_new(in, gr, k));
    rhoge = rhoge + (tmp2 - tmp);
  }
  T rq[6], q[6];
#pragma unroll
  for (int n = 0; n < 6; ++n) rq[n] = in.w(W_RQ_N + n, k);
#pragma unroll
  for (int n = 0; n < 6; ++n) q[n] = div_rn(rq[n], rhog, rrhog);
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
  // SATURATION_adjustment (mod_satadjust.cpp:274-362); with the switch
  // explicit_icegen = 0 cloud ice joins it (satadjust_all)
  const bool ice_adj = P.opt && C.opt_expice == 0.0;
  T ein_moist, qsum;
  if (ice_adj) {
    ein_moist = ein + q[I_QV] * LHV0 - q[I_QI] * LHF0;
    qsum = q[I_QV] + q[I_QC] + q[I_QI];
    q[I_QI] = T(0.0);
  } else {
    ein_moist = ein + q[I_QV] * LHV0;
    qsum = q[I_QV] + q[I_QC];
  }
  q[I_QV] = qsum;
  q[I_QC] = T(0.0);
  T cvtot = qd * CVDRY;
#pragma unroll
  for (int n = 1; n <= 5; ++n) cvtot = cvtot + q[n] * CVDRY;
  const T rho_l = rho;
  tem = (ein_moist - q[I_QV] * LHV0) / cvtot;
  int rc = 0;
  if (interior)
    rc = ice_adj ? satadjust_all_t(C, fm, P.itelim, ein_moist, qsum, rho_l, q, tem, iters)
                 : satadjust_t(C, fm, P.itelim, ein_moist, qsum, rho_l, q, tem, iters);
  rq[I_QV] = rhog * q[I_QV];
  rq[I_QC] = rhog * q[I_QC];
  if (ice_adj) rq[I_QI] = rhog * q[I_QI];
  cvtot = qd * CVDRY;
#pragma unroll
  for (int n = 1; n <= 5; ++n) cvtot = cvtot + q[n] * CVDRY;
  rhoge = rhog * tem * cvtot;
  T rhog_o = rhog;
  if (interior) {
    // negative_filter (mod_mp_nsw6.cpp:1770-1831)
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
  fin(SF_RHOG, rhog_o);
  fin(SF_RHOGE, rhoge);
#pragma unroll
  for (int n = 0; n < 6; ++n) {
    fin(SF_RQ + n, rq[n]);
    fin(SF_Q + n, q[n]);
  }
  fin(SF_RHO, rho);
  fin(SF_TEM, tem);
  fin(SF_PRE, pre);
  fin(SF_QD, qd);
  return rc;
}

__device__ __forceinline__ void stage_smem(const Problem& P, double* grid, double* tab) {
  for (int c = threadIdx.x; c < GF_COUNT * P.kall; c += blockDim.x) grid[c] = P.grid[c];
  for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = P.fmtab[c];
  __syncthreads();
}

__device__ __forceinline__ void tape_bind_s(const TapeMem& tm) {
  Tape& t = tape();
  t.pa = tm.pa;
  t.pb = tm.pb;
  t.da = tm.da;
  t.db = tm.db;
  t.adj = tm.adj;
  t.nslot = tm.nslot;
  t.slot = blockIdx.x * blockDim.x + threadIdx.x;
  t.cap = tm.cap;
  t.count_only = 0;
}

// Starts a new record on the calling thread's tape.
__device__ __forceinline__ void tape_begin(LeafLog& lg) {
  Tape& t = tape();
  t.n = 0;
  t.overflow = 0;
  lg.n = 0;
  lg.overflow = 0;
}

// Zeroes the adjoints of the recorded entries (after seeding nothing yet).
__device__ __forceinline__ void tape_clear_adj() {
  Tape& t = tape();
  for (int e = 0; e < t.n; ++e) t.adj[(size_t)e * t.nslot + t.slot] = 0.0;
}

__device__ __forceinline__ void seed(const RVar& v, double g) {
  if (v.id >= 0 && g != 0.0) adj_of(v) += g;
}

// Adds the adjoints of the logged leaves to where their values came from.
__device__ __forceinline__ void scatter(const StageIO& io, const LeafLog& lg) {
  for (int e = 0; e < lg.n; ++e) {
    const double g = adj_of(RVar(0.0, lg.id[e]));
    if (g == 0.0) continue;
    const int kind = lg.code[e] / 4096, f = lg.code[e] % 4096;
    double* dst = kind == LK_W ? io.WB + f * io.NC : kind == LK_Y ? io.YB + f * io.NC : io.xb.a[f];
    atomicAdd(dst + lg.idx[e], g);
  }
}

// Reports a stage whose tape or leaf log ran out of room.
__device__ __forceinline__ bool stage_overflow(const StageIO& io, const LeafLog& lg, int k, int g, int l) {
  if (tape().overflow || lg.overflow) {
    record_err(io.P.status, ERR_ADJ_CAPACITY, k, g, l, tape().n);
    return true;
  }
  return false;
}

// ------------------------------------------------------------------ kernels
// Flux bounds kcell_min / kcell_max of every region, row and level from the
// departure-distance extrema (mod_vadv1d.cpp:316-353), one thread each, as
// the column kernel forms them.
__global__ void adj_bounds_kernel(Problem P, int* bnd) {
  const int K = P.kall;
  const int nrow = 2 * P.ntr;
  const int n = P.lall * nrow * K;
  const double* gzh = P.grid + GF_GZH * K;
  const double* gzs = P.grid + GF_GZSHIFT * K;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int k = e % K, s = (e / K) % nrow, l = e / (nrow * K);
    const int half = s / P.ntr;
    const int mkmin = half ? P.kmin + 1 : P.kmin;
    const double* zh = half ? gzs : gzh;
    int lo = k, hi = k;
    if (k >= mkmin && k <= P.kmax) {
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
            lo = k2;
            break;
          }
      }
      if (zzmin < 0.0) {
        for (int k2 = k; k2 <= P.kmax; ++k2)
          if ((zh[k2] <= zh[k] - zzmin) && (zh[k2 + 1] > zh[k] - zzmin)) {
            hi = k2;
            break;
          }
      }
    }
    bnd[((size_t)l * 2 + 0) * 2 * MAX_TR * K + s * K + k] = lo;
    bnd[((size_t)l * 2 + 1) * 2 * MAX_TR * K + s * K + k] = hi;
  }
}

// Forward of S1.  A block is STAGE_THREADS columns of one level of one region
// (grid: columns, levels, regions), so that the per-level extrema of the
// departure distances over the region (vadv1d_prep, mod_vadv1d.cpp:316-353)
// reduce within the block: one 64-bit atomic per block and row, on
// order-preserving keys (exact, independent of the order of the atomics).
template <bool MIX>
__global__ void __launch_bounds__(STAGE_THREADS) adj_s1_fwd_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  __shared__ float grf[MIX ? 4 * MAX_KALL : 1];   // MIX: rdgz, rdgzh, rdzs, rdzsh in FP32
  __shared__ unsigned long long red[2][2 * MAX_TR][STAGE_THREADS / 32];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  if constexpr (MIX) {
    const int rows[4] = {GF_RDGZ, GF_RDGZH, GF_RDZS, GF_RDZSH};
    for (int c = threadIdx.x; c < 4 * io.P.kall; c += blockDim.x)
      grf[c] = (float)io.P.grid[rows[c / io.P.kall] * io.P.kall + c % io.P.kall];
  }
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y, l = blockIdx.z;
  const bool valid = g < io.L.G;
  const int nrow = 2 * io.P.ntr;
  double z[2 * MAX_TR] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (valid) {
    const size_t c = io.L.f(l, k, g);
    const In<double> in{io, l, g};
    stage1<double, MIX>(
        in, grid, k,
        [&](int f, double v) {
          io.W[f * io.NC + c] = v;
          if (f < nrow) z[f] = v;
        },
        grf);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int r = 0; r < nrow; ++r) {
    const int mkmin = r < io.P.ntr ? io.P.kmin : io.P.kmin + 1;
    const bool in_range = valid && k >= mkmin && k <= io.P.kmax && z[r] == z[r];   // NaN never wins
    unsigned long long kmx = in_range ? order_key(z[r]) : 0ull;
    unsigned long long kmn = in_range ? order_key(z[r]) : ~0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long a = __shfl_xor_sync(0xffffffffu, kmx, o);
      const unsigned long long b = __shfl_xor_sync(0xffffffffu, kmn, o);
      kmx = a > kmx ? a : kmx;
      kmn = b < kmn ? b : kmn;
    }
    if (lane == 0) {
      red[0][r][wid] = kmx;
      red[1][r][wid] = kmn;
    }
  }
  __syncthreads();
  if (threadIdx.x < nrow) {
    const int r = threadIdx.x;
    unsigned long long kmx = 0ull, kmn = ~0ull;
    for (int w = 0; w < (int)blockDim.x / 32; ++w) {
      kmx = red[0][r][w] > kmx ? red[0][r][w] : kmx;
      kmn = red[1][r][w] < kmn ? red[1][r][w] : kmn;
    }
    const size_t e = ((size_t)l * nrow + r) * io.P.kall + k;
    if (kmx != 0ull) atomicMax(&io.P.zmax[e], kmx);
    if (kmn != ~0ull) atomicMin(&io.P.zmin[e], kmn);
  }
}

// Forward of S2 (a work item per cell and flux).
__global__ void __launch_bounds__(STAGE_THREADS) adj_s2_fwd_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  __syncthreads();
  const int nj = 8 * io.P.ntr;
  for (int j = 0; j < nj; ++j)
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < io.NC; c += (size_t)gridDim.x * blockDim.x) {
      int g, k, l;
      io.L.split(c, l, k, g);
      const In<double> in{io, l, g};
      io.W[(W_F + j) * io.NC + c] = stage2<double>(in, grid, k, j);
    }
}

// Forward of S3.
__global__ void __launch_bounds__(STAGE_THREADS) adj_s3_fwd_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  __syncthreads();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < io.NC; c += (size_t)gridDim.x * blockDim.x) {
    int g, k, l;
    io.L.split(c, l, k, g);
    const In<double> in{io, l, g};
    stage3<double>(
        in, grid, k, [&](int f, double v) { io.W[f * io.NC + c] = v; }, [](int, double) {}, [](int, double) {});
  }
}

// Adjoint of S4, recorded on a tape (adjoint mode 1): seeds from the caller's output adjoints.
__global__ void __launch_bounds__(STAGE_THREADS) adj_s4_kernel(StageIO io, Consts C, TapeMem tm) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  __shared__ double tab[FM_TABLE_DOUBLES];
  stage_smem(io.P, grid, tab);
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  tape_bind_s(tm);
  LeafLog lg;
  for (size_t c = tape().slot; c < io.NC; c += tape().nslot) {
    int g, k, l;
    io.L.split(c, l, k, g);
    tape_begin(lg);
    const In<RVar> in{io, l, g, &lg};
    RVar outs[NSF];
    int it = 0;
    const int rc = stage4<RVar>(in, C, grid, fm, k, [&](int f, const RVar& v) { outs[f] = v; }, &it);
    if (rc) record_err(io.P.status, rc, k, g, l, it);
    if (stage_overflow(io, lg, k, g, l)) continue;
    tape_clear_adj();
    for (int f = 0; f < NSF; ++f) {
      const bool momentum = f == SF_RVX || f == SF_RVY || f == SF_RVZ || f == SF_RW;
      if (f != SF_GPREC && (!momentum || io.kin2kin)) seed(outs[f], io.SB[f * io.NC + c]);
    }
    tape_reverse();
    scatter(io, lg);
    if (io.kin2kin) {
      // consumed here: the S3 sweep adds the momentum seeds only without KIN2KIN
      double* SB = const_cast<double*>(io.SB);
      SB[SF_RVX * io.NC + c] = SB[SF_RVY * io.NC + c] = SB[SF_RVZ * io.NC + c] = SB[SF_RW * io.NC + c] = 0.0;
    }
  }
}

// Adjoint of S4, hand-written: the cell's forward (KIN2EIN, thermodynamics,
// saturation adjustment, negative filter) recomputed as stage4 does, then the
// reverse sweep.  The Newton temperature is differentiated implicitly at its
// converged value as satadjust_t does: with F(T) = T cv(T) + qsat(T) LHV0 -
// Emoist, dT = -dF / F_T at the last iterate.  Adjoints go to S3's outputs at
// this level and its neighbours and to the metric factors, atomically.
__global__ void __launch_bounds__(STAGE_THREADS) adj_s4_hw_kernel(StageIO io, Consts C, int pass) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  __shared__ double tab[FM_TABLE_DOUBLES];
  stage_smem(io.P, grid, tab);
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  const Problem& P = io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const double* afact = grid + GF_AFACT * K;
  const double* bfact = grid + GF_BFACT * K;
  const double* cfact = grid + GF_CFACT * K;
  const double* dfact = grid + GF_DFACT * K;
  const size_t NC = io.NC;
  const size_t G = io.L.G;
  auto cell = [&](const size_t c, const bool first) {
    int g, k, l;
    io.L.split(c, l, k, g);
    const bool interior = (k >= kmin && k <= kmax);
    auto W = [&](int f, size_t cc) { return io.W[f * NC + cc]; };
    auto WBadd = [&](int f, size_t cc, double v) {
      if (!fp_is_zero(v)) atomicAdd(&io.WB[f * NC + cc], v);
    };
    auto XBadd = [&](int a, size_t i, double v) {
      if (!fp_is_zero(v)) atomicAdd(&io.xb.a[a][i], v);
    };
    const double* gs = io.x.a[A_gsgam2];
    const double* gsh = io.x.a[A_gsgam2h];
    // ------------------------------------------------------------ forward
    const double rhog = W(W_RHOG_N, c);
    const double rrhog = 1.0 / rhog;
    const double rhoge_a = W(W_RHOGE_N, c);
    const double gsg = gs[c];
    const double rgsg = 1.0 / gsg;   // the reciprocals of gsgam2 at k - 1, k, k + 1 serve both sweeps
    double rg_up = 0.0, rg_dn = 0.0;
    double rhoge = rhoge_a;
    // KIN2EIN pieces
    double gh = 0, rgh = 0, w2c0 = 0, w2c1 = 0, kinh = 0, kvp = 0, kv0 = 0, rvx = 0, rvy = 0, rvz = 0, tmp_h = 0;
    double kvu[2] = {0, 0}, den[2] = {0, 0}, c2a[2] = {0, 0}, c2b[2] = {0, 0}, rwj[2] = {0, 0};
    bool hv[2] = {false, false};
    if (interior) {
      gh = gsh[c + G];
      rgh = 1.0 / gh;
      w2c0 = div_rn(cfact[k] * gsg, gh, rgh);
      w2c1 = div_rn(dfact[k] * gsg, gh, rgh);
      kinh = W(W_KINH_N, c);
      kvp = W(W_KINV_N, c + G);
      kv0 = W(W_KINV_N, c);
      const double tmp2 = kinh + (w2c0 * kvp + w2c1 * kv0);
      rvx = W(W_RVX_N, c);
      rvy = W(W_RVY_N, c);
      rvz = W(W_RVZ_N, c);
      tmp_h = div_rn(0.5 * (rvx * rvx + rvy * rvy + rvz * rvz), rhog, rrhog);
      for (int s2 = 0; s2 < 2; ++s2) {   // s2 = 0: level k + 1, 1: level k
        const int j = k + 1 - s2;
        const size_t cj = c + G - s2 * G;
        hv[s2] = (j >= kmin + 1 && j <= kmax);
        if (!hv[s2]) continue;
        const double ghj = gsh[cj];
        // afact / gs(j) and bfact / gs(j-1), correctly rounded, from the reciprocals
        if (s2 == 0) rg_up = 1.0 / gs[cj];
        else rg_dn = 1.0 / gs[cj - G];
        const double rgj = s2 == 0 ? rg_up : rgsg, rgjm = s2 == 0 ? rgsg : rg_dn;
        c2a[s2] = div_rn(afact[j], gs[cj], rgj) * ghj;
        c2b[s2] = div_rn(bfact[j], gs[cj - G], rgjm) * ghj;
        rwj[s2] = W(W_RW_N, cj);
        den[s2] = c2a[s2] * W(W_RHOG_N, cj) + c2b[s2] * W(W_RHOG_N, cj - G);
        kvu[s2] = 0.5 * (rwj[s2] * rwj[s2]) / den[s2];
      }
      const double tmp = tmp_h + (w2c0 * kvu[0] + w2c1 * kvu[1]);
      rhoge = rhoge_a + (tmp2 - tmp);
    }
    double rq[6], qo[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) rq[n] = W(W_RQ_N + n, c);
#pragma unroll
    for (int n = 0; n < 6; ++n) qo[n] = div_rn(rq[n], rhog, rrhog);
    const double rho1 = rhog / gsg;
    const double ein = div_rn(rhoge, rhog, rrhog);
    double qd = 1.0;
#pragma unroll
    for (int n = 1; n <= 5; ++n) qd = qd - qo[n];
    // THRMDYN_tempre (its pressure is an output at the halo levels)
    double cvt = 0.0, qdl = 1.0;
#pragma unroll
    for (int n = 1; n <= 5; ++n) {
      cvt = cvt + qo[n] * CVDRY;
      qdl = qdl - qo[n];
    }
    cvt = cvt + qdl * CVDRY;
    const double tem0 = ein / cvt;
    const double pq0 = qdl * RDRY + qo[0] * RVAP;
    const double ein_moist = ein + qo[0] * LHV0;
    const double qsum = qo[0] + qo[1];
    double q[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) q[n] = qo[n];
    q[0] = qsum;
    q[1] = 0.0;
    double cvtot1 = qd * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cvtot1 = cvtot1 + q[n] * CVDRY;
    const double tem_p = (ein_moist - q[0] * LHV0) / cvtot1;
    double tem = tem_p;
    // saturation adjustment (satadjust_t's iteration, then its implicit derivative pieces)
    bool sat = false;
    double ts = 0, qsT = 0, cvT = 0, FT = 0, dqs = 0, qd_l = 0;
    int sc = 0;
    if (interior) {
      qd_l = 1.0;
#pragma unroll
      for (int n = 1; n <= 5; ++n) qd_l = qd_l - q[n];
      // the test decided in FP32 where its margin allows (sat_screen_liq)
      sc = sat_screen_liq(tem, rho1, qsum, float(C.LovR_liq));
      if (sc < 0) {
        const double rtem0 = 1.0 / fp_max_pos(tem, TEM_MIN);
        const double psat0 = PSAT0 * fm.exp(C.LovR_liq * (C.RTEM00 - rtem0));
        sc = (qsum - psat0 / (rho1 * RVAP * tem) > EPS) ? 1 : 0;
      }
    }
    if (first) {
      // A saturated cell goes to the list of the second pass, whose warps it
      // fills: here its Newton iteration would hold its level's whole warp.
      // One atomic per warp on the list's count.
      const unsigned m = __activemask();
      const unsigned b = __ballot_sync(m, sc != 0);
      if (b) {
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        unsigned base = 0u;
        if (lane == leader) base = atomicAdd(io.P.satq, (unsigned)__popc(b));
        base = __shfl_sync(m, base, leader);
        if (sc) io.P.satq[1 + base + __popc(b & ((1u << lane) - 1u))] = (unsigned)c;
      }
      if (sc) return;
    }
    if (interior) {
      double tv = tem;
      if (sc) {
        double qv[6];
#pragma unroll
        for (int n = 0; n < 6; ++n) qv[n] = q[n];
        bool converged = false;
        double tprev = tv, qs_last = 0.0;
        int ite;
        for (ite = 0; ite < P.itelim; ++ite) {
          tprev = tv;
          const double rtem = 1.0 / fp_max_pos(tv, TEM_MIN);
          const double psat = PSAT0 * fm.exp(C.LovR_liq * (C.RTEM00 - rtem));
          const double qsat = psat / (rho1 * RVAP * tv);
          qs_last = qsat;
          qv[I_QV] = qsat;
          qv[I_QC] = qsum - qsat;
          double cv = qd_l * CVDRY;
#pragma unroll
          for (int n = 1; n <= 5; ++n) cv = cv + qv[n] * CVDRY;
          const double emoist_new = tv * cv + qv[I_QV] * LHV0;
          const double dqsat_dT = C.LovR_liq * rtem * rtem * qsat;
          const double demoist_dT = cv + dqsat_dT * LHV0;
          const double dtemp = (emoist_new - ein_moist) / demoist_dT;
          tv = tv - dtemp;
          if (fp_abs_lt(dtemp, C.dtemp_criteria)) {
            converged = true;
            break;
          }
          if (fp_not_finite(tv)) break;
        }
        tem = tv;
        q[I_QV] = qv[I_QV];
        q[I_QC] = qv[I_QC];
        if (converged) {
          sat = true;
          ts = tprev;
          qsT = qs_last;   // qsat at the last iterate ts, as the iteration formed it
          cvT = qd_l * CVDRY + (qsum - qsT) * CVDRY;
#pragma unroll
          for (int n = 2; n <= 5; ++n) cvT = cvT + q[n] * CVDRY;
          const double rts = 1.0 / ts;
          dqs = qsT * (C.LovR_liq * rts * rts - rts);
          FT = cvT - ts * dqs * CVDRY + dqs * LHV0;
        } else {
          record_err(P.status, fp_not_finite(tv) ? 4 : 3, k, g, l, ite);
        }
      }
    }
    double rq2[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) rq2[n] = rq[n];
    rq2[I_QV] = rhog * q[I_QV];
    rq2[I_QC] = rhog * q[I_QC];
    double cvtot2 = qd * CVDRY;
#pragma unroll
    for (int n = 1; n <= 5; ++n) cvtot2 = cvtot2 + q[n] * CVDRY;
    // negative filter (interior)
    bool clip[6] = {false, false, false, false, false, false};
    double rqf[6], qf[6], d2 = 0, rhog_o = rhog, rrhog_o = rrhog, rho_f = 0, qdf = 0, cva = 0, pq_f = 0;
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      rqf[n] = rq2[n];
      qf[n] = q[n];
    }
    if (interior) {
      double diffq = 0.0;
#pragma unroll
      for (int n = 2; n <= 5; ++n) {
        diffq += rqf[n];
        clip[n] = lt_z(rqf[n]);
        rqf[n] = clip[n] ? 0.0 : rqf[n];
      }
#pragma unroll
      for (int n = 2; n <= 5; ++n) diffq -= rqf[n];
      rqf[0] += diffq;
      d2 = rqf[0];
      clip[0] = lt_z(rqf[0]);
      rqf[0] = clip[0] ? 0.0 : rqf[0];
      d2 -= rqf[0];
      if (fp_is_zero(d2) && fp_pos_normal(rhog)) {
        // nothing removed: rhog (1 - d2) = rhog exactly, rho_f = rho1 and the
        // reciprocal as above, and the quotients of the tracers the filter left
        // as they were are q's (q[QC] is +0 unless the iteration ran)
        rho_f = rho1;
#pragma unroll
        for (int n = 1; n <= 5; ++n)
          if (n == I_QC ? fp_bits(q[I_QC]) != 0 : clip[n]) qf[n] = div_rn(rqf[n], rhog, rrhog);
      } else {
        rhog_o = rhog * (1.0 - d2);
        rho_f = rhog_o / gsg;
        rrhog_o = 1.0 / rhog_o;
#pragma unroll
        for (int n = 1; n <= 5; ++n) qf[n] = div_rn(rqf[n], rhog_o, rrhog_o);
      }
      qdf = 1.0;
#pragma unroll
      for (int n = 1; n <= 5; ++n) qdf = qdf - qf[n];
      cva = qdf * CVDRY;
#pragma unroll
      for (int n = 1; n <= 5; ++n) cva = cva + qf[n] * CVDRY;
      pq_f = qdf * RDRY + qf[I_QV] * RVAP;
    }
    // ------------------------------------------------------------ reverse
    // (divisions by reciprocals: the adjoint's coefficients need no correct rounding)
    const double* SB = io.SB;
    double b_tem = SB[SF_TEM * NC + c];
    double b_qd = SB[SF_QD * NC + c];
    double b_q[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) b_q[n] = SB[(SF_Q + n) * NC + c];
    double b_rq2[6];
    double b_rhog = 0.0, b_rho1 = 0.0, b_pre0 = 0.0, b_rhoge2 = 0.0, b_gsg = 0.0;
    if (interior) {
      const double B_pre = SB[SF_PRE * NC + c], B_rhoge = SB[SF_RHOGE * NC + c];
      double b_rhog_o = SB[SF_RHOG * NC + c];
      // pre = ((rho_f pq_f) tem)
      b_tem += B_pre * rho_f * pq_f;
      double b_rho_f = SB[SF_RHO * NC + c] + B_pre * tem * pq_f;
      const double b_pq = B_pre * tem * rho_f;
      double b_qdf = b_pq * RDRY;
      b_q[I_QV] += b_pq * RVAP;
      // rhoge = (tem rhog_o) cva
      b_tem += B_rhoge * rhog_o * cva;
      b_rhog_o += B_rhoge * tem * cva;
      const double b_cva = B_rhoge * tem * rhog_o;
      b_qdf += b_cva * CVDRY;
      double b_qf[6];
#pragma unroll
      for (int n = 1; n <= 5; ++n) b_qf[n] = b_q[n] + b_cva * CVDRY - b_qdf;
      // qf = rqf / rhog_o; rho_f = rhog_o / gsg
      double b_rqf[6];
#pragma unroll
      for (int n = 0; n < 6; ++n) b_rqf[n] = SB[(SF_RQ + n) * NC + c];
#pragma unroll
      for (int n = 1; n <= 5; ++n) {
        b_rqf[n] += b_qf[n] * rrhog_o;
        b_rhog_o -= b_qf[n] * qf[n] * rrhog_o;
      }
      b_rhog_o += b_rho_f * rgsg;
      b_gsg -= b_rho_f * rho_f * rgsg;
      // rhog_o = rhog (1 - d2)
      b_rhog += b_rhog_o * (1.0 - d2);
      const double b_d2 = -b_rhog_o * rhog;
      const double b_rq0a = (clip[0] ? b_d2 : 0.0) + (clip[0] ? 0.0 : b_rqf[0]);
      b_rq2[0] = b_rq0a;
      b_rq2[1] = b_rqf[1];
#pragma unroll
      for (int n = 2; n <= 5; ++n) b_rq2[n] = (clip[n] ? b_rq0a : 0.0) + (clip[n] ? 0.0 : b_rqf[n]);
      // the q outputs are the filter's for n >= 1: their adjoints were taken above
#pragma unroll
      for (int n = 1; n <= 5; ++n) b_q[n] = 0.0;
    } else {
#pragma unroll
      for (int n = 0; n < 6; ++n) b_rq2[n] = SB[(SF_RQ + n) * NC + c];
      b_rhoge2 = SB[SF_RHOGE * NC + c];
      b_rhog += SB[SF_RHOG * NC + c];
      b_rho1 += SB[SF_RHO * NC + c];
      b_pre0 = SB[SF_PRE * NC + c];
    }
    // rhoge2 = (rhog tem) cvtot2 (the output at the halo levels)
    if (!fp_is_zero(b_rhoge2)) {
      b_rhog += b_rhoge2 * tem * cvtot2;
      b_tem += b_rhoge2 * rhog * cvtot2;
      const double b_cv2 = b_rhoge2 * rhog * tem;
      b_qd += b_cv2 * CVDRY;
#pragma unroll
      for (int n = 1; n <= 5; ++n) b_q[n] += b_cv2 * CVDRY;
    }
    // rq2[QV] = rhog q[QV], rq2[QC] = rhog q[QC]; rq2[n >= 2] = rq[n]
    b_rhog += b_rq2[I_QV] * q[I_QV] + b_rq2[I_QC] * q[I_QC];
    b_q[I_QV] += b_rq2[I_QV] * rhog;
    b_q[I_QC] += b_rq2[I_QC] * rhog;
    double b_rq[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int n = 2; n <= 5; ++n) b_rq[n] += b_rq2[n];
    // saturation adjustment
    double b_ein_moist = 0.0, b_qsum = 0.0, b_rho_l = 0.0, b_tem_p = 0.0, b_q0p = 0.0;
    if (sat) {
      const double b_qc = b_q[I_QC], b_qv = b_q[I_QV];
      b_qsum += b_qc;
      const double b_qsI = b_qv - b_qc;
      double b_qsT = b_qsI;
      const double b_temI = b_tem + b_qsI * dqs;
      const double b_F = -b_temI * (1.0 / FT);
      const double b_cvT = b_F * ts;
      b_qsT += b_F * LHV0;
      b_ein_moist -= b_F;
      const double b_qd_l = b_cvT * CVDRY;
      b_qsum += b_cvT * CVDRY;
      b_qsT -= b_cvT * CVDRY;
#pragma unroll
      for (int n = 2; n <= 5; ++n) b_q[n] += b_cvT * CVDRY - b_qd_l;
      b_rho_l -= b_qsT * qsT * (gsg * rrhog);
    } else {
      b_tem_p = b_tem;
      b_q0p = b_q[I_QV];
    }
    // tem_p = (ein_moist - qsum LHV0) / cvtot1, cvtot1 = qd CV + sum_{n >= 2} q[n] CV
    {
      const double rcv1 = 1.0 / cvtot1;
      const double b_num = b_tem_p * rcv1;
      const double b_cv1 = -b_tem_p * tem_p * rcv1;
      b_ein_moist += b_num;
      b_qsum -= b_num * LHV0;
      b_qd += b_cv1 * CVDRY;
#pragma unroll
      for (int n = 2; n <= 5; ++n) b_q[n] += b_cv1 * CVDRY;
    }
    b_qsum += b_q0p;
    b_rho1 += b_rho_l;
    // q[n >= 2] = qo[n]; qsum = qo[0] + qo[1]; ein_moist = ein + qo[0] LHV0
    double b_qo[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) b_qo[n] = (n >= 2) ? b_q[n] : 0.0;
    b_qo[0] += b_qsum + b_ein_moist * LHV0;
    b_qo[1] += b_qsum;
    double b_ein = b_ein_moist;
    // pre0 = (rho1 tem0) pq0 (halo output)
    if (!fp_is_zero(b_pre0)) {
      b_rho1 += b_pre0 * tem0 * pq0;
      const double b_tem0 = b_pre0 * rho1 * pq0;
      const double b_pq0 = b_pre0 * rho1 * tem0;
      const double b_qdl0 = b_pq0 * RDRY;
      b_qo[0] += b_pq0 * RVAP;
      const double rcvt = 1.0 / cvt;
      b_ein += b_tem0 * rcvt;
      const double b_cvt = -b_tem0 * tem0 * rcvt;
      const double b_qdl = b_qdl0 + b_cvt * CVDRY;
#pragma unroll
      for (int n = 1; n <= 5; ++n) b_qo[n] += b_cvt * CVDRY - b_qdl;
    }
    // qd = 1 - sum qo[1..5]
#pragma unroll
    for (int n = 1; n <= 5; ++n) b_qo[n] -= b_qd;
    // ein = rhoge / rhog, rho1 = rhog / gsg, qo = rq / rhog
    double b_rhoge = b_ein * rrhog;
    b_rhog -= b_ein * ein * rrhog;
    b_rhog += b_rho1 * rgsg;
    b_gsg -= b_rho1 * rho1 * rgsg;
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      b_rq[n] += b_qo[n] * rrhog;
      b_rhog -= b_qo[n] * qo[n] * rrhog;
    }
    // KIN2EIN
    if (interior) {
      const double b_tmp2 = b_rhoge, b_tmp = -b_rhoge;
      WBadd(W_KINH_N, c, b_tmp2);
      WBadd(W_KINV_N, c + G, b_tmp2 * w2c0);
      WBadd(W_KINV_N, c, b_tmp2 * w2c1);
      double b_w2c0 = b_tmp2 * kvp + b_tmp * kvu[0];
      double b_w2c1 = b_tmp2 * kv0 + b_tmp * kvu[1];
      const double b_tmp_h = b_tmp;
      const double b_sq = b_tmp_h * rrhog;
      b_rhog -= b_tmp_h * tmp_h * rrhog;
      WBadd(W_RVX_N, c, b_sq * rvx);
      WBadd(W_RVY_N, c, b_sq * rvy);
      WBadd(W_RVZ_N, c, b_sq * rvz);
      for (int s2 = 0; s2 < 2; ++s2) {
        if (!hv[s2]) continue;
        const int j = k + 1 - s2;
        const size_t cj = c + G - s2 * G;
        const double b_kvu = b_tmp * (s2 == 0 ? w2c0 : w2c1);
        const double rden = 1.0 / den[s2];
        WBadd(W_RW_N, cj, b_kvu * rwj[s2] * rden);
        const double b_den = -b_kvu * kvu[s2] * rden;
        WBadd(W_RHOG_N, cj, b_den * c2a[s2]);
        WBadd(W_RHOG_N, cj - G, b_den * c2b[s2]);
        const double b_c2a = b_den * W(W_RHOG_N, cj), b_c2b = b_den * W(W_RHOG_N, cj - G);
        // c2a = (afact / gs(j)) gsh(j), c2b = (bfact / gs(j-1)) gsh(j)
        const double rgj = s2 == 0 ? rg_up : rgsg, rgjm = s2 == 0 ? rgsg : rg_dn;
        XBadd(A_gsgam2h, cj, b_c2a * (afact[j] * rgj) + b_c2b * (bfact[j] * rgjm));
        XBadd(A_gsgam2, cj, -b_c2a * c2a[s2] * rgj);
        XBadd(A_gsgam2, cj - G, -b_c2b * c2b[s2] * rgjm);
      }
      // w2c0 = cfact gsg / gh, w2c1 = dfact gsg / gh
      b_gsg += (b_w2c0 * cfact[k] + b_w2c1 * dfact[k]) * rgh;
      XBadd(A_gsgam2h, c + G, -(b_w2c0 * w2c0 + b_w2c1 * w2c1) * rgh);
      WBadd(W_RHOGE_N, c, b_rhoge);
    } else {
      WBadd(W_RHOGE_N, c, b_rhoge);
    }
    WBadd(W_RHOG_N, c, b_rhog);
#pragma unroll
    for (int n = 0; n < 6; ++n) WBadd(W_RQ_N + n, c, b_rq[n]);
    XBadd(A_gsgam2, c, b_gsg);
  };
  if (pass == 0) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < NC; c += (size_t)gridDim.x * blockDim.x)
      cell(c, true);
  } else {
    const unsigned n = io.P.satq[0];
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
      cell(io.P.satq[1 + e], false);
  }
}

// Adjoint of vadv_zdis_wh at level k: the adjoints of wh(k-1), wh(k), wh(k+1)
// (bw[0..2]) from that of zdis.  At k == mkmin only wh(k) and wh(k+1) enter.
template <class R>
__device__ __forceinline__ void zdis_wh_bar(R wm, R w0, R wpp, const R* rdz, const R* rdzs, int k, int mkmin, R dt,
                                            R hdt2, R sdt3, R bz, R* bw) {
  if (k == mkmin) {
    // z = (-hdt2 w0) ((wpp - w0) rdz) + dt w0
    const R a = -hdt2 * w0, b = (wpp - w0) * rdz[mkmin];
    bw[0] = R(0.0);
    bw[1] = bz * (-hdt2 * b - a * rdz[mkmin] + dt);
    bw[2] = bz * a * rdz[mkmin];
    return;
  }
  const R rs = rdzs[k];
  const R r = (wpp - wm) * rs;
  const R c = R(2.0) * rs * ((wpp - w0) * rdz[k] - (w0 - wm) * rdz[k - 1]);
  // z = (-hdt2 w0) r + dt w0 + (sdt3 w0) (w0 c + r r)
  const R b_r = bz * (-hdt2 * w0 + sdt3 * w0 * R(2.0) * r);
  const R b_c = bz * sdt3 * w0 * w0;
  R b_w0 = bz * (-hdt2 * r + dt + sdt3 * (R(2.0) * w0 * c + r * r));
  const R b_d = b_c * R(2.0) * rs;
  b_w0 = fmaR(-b_d, (rdz[k] + rdz[k - 1]), b_w0);
  bw[0] = -b_r * rs + b_d * rdz[k - 1];
  bw[1] = b_w0;
  bw[2] = b_r * rs + b_d * rdz[k];
}

// Adjoint of S1, hand-written: the cell's departure distances, kinetic
// energies and flux sources recomputed as stage1 does, then the reverse
// sweep.  Only interior cells have non-constant outputs.  Adjoints of values
// at this cell that no other thread of the launch touches are added in place;
// those at level k - 1, of the fall speeds at k - 3 .. k + 1 and of the
// column's unit vectors go by atomics.
// MIX: the departure distances are the mixed step's (FP32, stage1): their
// adjoint coefficients in FP32 at the FP32 values, times the FP64 adjoint.
template <bool MIX>
__global__ void __launch_bounds__(STAGE_THREADS) adj_s1_hw_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  __shared__ float grf[MIX ? 4 * MAX_KALL : 1];   // MIX: rdgz, rdgzh, rdzs, rdzsh in FP32
  for (int i = threadIdx.x; i < GF_COUNT * io.P.kall; i += blockDim.x) grid[i] = io.P.grid[i];
  if constexpr (MIX) {
    const int rows[4] = {GF_RDGZ, GF_RDGZH, GF_RDZS, GF_RDZSH};
    for (int c = threadIdx.x; c < 4 * io.P.kall; c += blockDim.x)
      grf[c] = (float)io.P.grid[rows[c / io.P.kall] * io.P.kall + c % io.P.kall];
  }
  __syncthreads();
  const Problem& P = io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const double* rdgz = grid + GF_RDGZ * K;
  const double* rdgzh = grid + GF_RDGZH * K;
  const double* rdzs = grid + GF_RDZS * K;
  const double* rdzsh = grid + GF_RDZSH * K;
  const double* afact = grid + GF_AFACT * K;
  const double* bfact = grid + GF_BFACT * K;
  const size_t NC = io.NC, G = io.L.G;
  const double dt = P.dt, hdt2 = P.hdt2, sdt3 = P.sdt3;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < NC; c += (size_t)gridDim.x * blockDim.x) {
    int g, k, l;
    io.L.split(c, l, k, g);
    if (k < kmin || k > kmax) continue;
    const bool hk = (k >= kmin + 1);
    const size_t cc = io.L.c(l, g);
    const double* const* x = io.x.a;
    double* const* xb = io.xb.a;
    auto Y = [&](int f, size_t i) { return io.Y[f * NC + i]; };
    auto YBadd = [&](int f, size_t i, double v) {
      if (!fp_is_zero(v)) atomicAdd(&io.YB[f * NC + i], v);
    };
    auto YBown = [&](int f, size_t i, double v) { io.YB[f * NC + i] += v; };
    auto XBadd = [&](int a, size_t i, double v) {
      if (!fp_is_zero(v)) atomicAdd(&xb[a][i], v);
    };
    auto XBown = [&](int a, size_t i, double v) { xb[a][i] += v; };
    auto WB = [&](int f) { return io.WB[f * NC + c]; };
    // ---------------------------------------------------- departure distances
    const int ntr = P.ntr;
    double vt[MAX_TR][5];
    for (int t = 0; t < ntr; ++t)
      for (int j = 0; j < 5; ++j) {
        const int kk = k - 3 + j;
        vt[t][j] = (kk >= kmin && kk <= kmax) ? Y(sed_tracer(t, ntr).vt, c + (size_t)(j - 3) * G) : 0.0;
      }
    double bvt[MAX_TR][5] = {};
    for (int r = 0; r < 2 * ntr; ++r) {
      const double bz = WB(W_ZDIS + r);
      if (fp_is_zero(bz)) continue;
      const int t = r % ntr, half = r / ntr;
      const int mkmin = half ? kmin + 1 : kmin;
      if (k < mkmin) continue;
      double bw[3];
      if constexpr (MIX) {
        auto col = [&](int j) { return float(vt[t][j - k + 3]); };
        auto wp = [&](int j) {
          if (!half) return col(j);
          return (j >= kmin + 1 && j <= kmax - 1) ? 0.5f * (col(j) + col(j - 1)) : 0.0f;
        };
        auto wh = [&](int j) { return vadv_wh<float>(wp, j, mkmin, kmax); };
        const float wm = k > mkmin ? wh(k - 1) : 0.0f;
        float cw[3];
        zdis_wh_bar<float>(wm, wh(k), wh(k + 1), grf + (half ? K : 0), grf + (half ? 3 * K : 2 * K), k, mkmin,
                           float(dt), float(hdt2), float(sdt3), 1.0f, cw);
        for (int i = 0; i < 3; ++i) bw[i] = bz * double(cw[i]);
      } else {
        auto col = [&](int j) { return vt[t][j - k + 3]; };
        auto wp = [&](int j) {
          if (!half) return col(j);
          return (j >= kmin + 1 && j <= kmax - 1) ? 0.5 * (col(j) + col(j - 1)) : 0.0;
        };
        auto wh = [&](int j) { return vadv_wh<double>(wp, j, mkmin, kmax); };
        const double wm = k > mkmin ? wh(k - 1) : 0.0;
        zdis_wh_bar<double>(wm, wh(k), wh(k + 1), half ? rdgzh : rdgz, half ? rdzsh : rdzs, k, mkmin, dt, hdt2,
                            sdt3, bz, bw);
      }
      auto add_wp = [&](int j, double v) {
        if (!half) {
          bvt[t][j - k + 3] += v;
        } else if (j >= kmin + 1 && j <= kmax - 1) {
          bvt[t][j - k + 3] += 0.5 * v;
          bvt[t][j - 1 - k + 3] += 0.5 * v;
        }
      };
      for (int s2 = 0; s2 < 3; ++s2) {
        const int j = k - 1 + s2;
        const double v = bw[s2];
        if (fp_is_zero(v)) continue;
        if (j >= mkmin + 1 && j <= kmax) {
          add_wp(j - 1, 0.5 * v);
          add_wp(j, 0.5 * v);
        } else if (j == mkmin) {
          add_wp(mkmin, v);
        } else if (j == mkmin - 1) {
          add_wp(mkmin - 1, v);
        } else {
          add_wp(kmax, v);
        }
      }
    }
    for (int t = 0; t < ntr; ++t)
      for (int j = 0; j < 5; ++j) {
        const int kk = k - 3 + j;
        if (kk >= kmin && kk <= kmax) YBadd(sed_tracer(t, ntr).vt, c + (size_t)(j - 3) * G, bvt[t][j]);
      }
    // ------------------------------------------- metric factors, kinetic energy
    // (recomputed for the partials only, so by reciprocals; no branch reads them)
    const size_t ck = c;   // (l, k, g) in the full-level fields
    const double gam2 = x[A_gam2][ck], gs = x[A_gsgam2][ck];
    const double rgsr = 1.0 / gs;
    const double rgs = gam2 * rgsr;
    const double vx = x[A_vx][ck], vy = x[A_vy][ck], vz = x[A_vz][ck];
    const double ix = x[A_ix][cc], iy = x[A_iy][cc], iz = x[A_iz][cc];
    const double jx = x[A_jx][cc], jy = x[A_jy][cc], jz = x[A_jz][cc];
    const double vi = vx * ix + vy * iy + vz * iz;
    const double vj = vx * jx + vy * jy + vz * jz;
    const double rvx = x[A_rhogvx][ck], rvy = x[A_rhogvy][ck], rvz = x[A_rhogvz][ck];
    const double rhog = Y(YS_RHOG, c);
    const double rrhog = 1.0 / rhog;
    const double kinh = 0.5 * (rvx * rvx + rvy * rvy + rvz * rvz) * rrhog;
    double gh = 0, rgh = 0, rgsm = 0, rden = 0, gsm = 0, c2w0 = 0, c2w1 = 0, rw = 0, rhogm = 0, den = 0, kinv = 0, gam2h = 0, rgsh = 0;
    if (hk) {
      gh = x[A_gsgam2h][ck];
      gsm = x[A_gsgam2][ck - G];
      rgh = 1.0 / gh;
      rgsm = 1.0 / gsm;
      c2w0 = afact[k] * rgsr * gh;
      c2w1 = bfact[k] * rgsm * gh;
      rw = x[A_rhogw][ck];
      rhogm = Y(YS_RHOG, c - G);
      den = c2w0 * rhog + c2w1 * rhogm;
      rden = 1.0 / den;
      kinv = 0.5 * (rw * rw) * rden;
      gam2h = x[A_gam2h][ck];
      rgsh = gam2h * rgh;
    }
    const double tem = Y(YS_TEM, c), zz = x[A_z][ck];
    // ------------------------------------------------------------- sources
    double b_kinh = WB(W_KINH), b_kinv = WB(W_KINV), b_rgs = 0.0, b_rgsh = 0.0, b_rw = 0.0;
    double b_tem = 0.0, b_zz = 0.0, b_vi = 0.0, b_vj = 0.0;
    for (int t = 0; t < ntr; ++t) {
      const int nq = sed_tracer(t, ntr).nq;
      const double* bs = io.WB + (size_t)(W_RHOF + 8 * t) * NC + c;
      const double b0 = bs[0], b1 = bs[NC], b2 = bs[2 * NC], b3 = bs[3 * NC], b4 = bs[4 * NC], b5 = bs[5 * NC];
      const double b6 = hk ? bs[6 * NC] : 0.0, b7 = hk ? bs[7 * NC] : 0.0;
      const double rq = Y(YS_RHOGQ + nq, c), qn = Y(YS_Q + nq - 1, c);
      const double base = rq * rgs;
      const double b_base = b0 + b1 * CVDRY * tem + b2 * GRAV * zz + b4 * vi + b5 * vj;
      b_tem = fma(b1 * base, CVDRY, b_tem);
      b_zz = fma(b2 * base, GRAV, b_zz);
      b_vi = fma(b4, base, b_vi);
      b_vj = fma(b5, base, b_vj);
      double b_qn = b3 * rgs * kinh;
      b_rgs += b3 * qn * kinh + b_base * rq;
      b_kinh = fma(b3 * qn, rgs, b_kinh);
      if (hk) {
        const double qm = Y(YS_Q + nq - 1, c - G);
        const double qh = 0.5 * (qn + qm) * rgsh;
        const double b_qh = b6 * kinv + b7 * rw;
        b_kinv = fma(b6, qh, b_kinv);
        b_rw = fma(b7, qh, b_rw);
        b_qn = fma(b_qh * 0.5, rgsh, b_qn);
        YBadd(YS_Q + nq - 1, c - G, b_qh * 0.5 * rgsh);
        b_rgsh = fma(b_qh * 0.5, (qn + qm), b_rgsh);
      }
      YBadd(YS_Q + nq - 1, c, b_qn);
      YBown(YS_RHOGQ + nq, c, b_base * rgs);
    }
    YBown(YS_TEM, c, b_tem);
    XBown(A_z, ck, b_zz);
    double b_rhog = 0.0, b_gs = 0.0;
    if (hk) {
      // rgsh = gam2h / gsgam2h; kinv = 0.5 rw^2 / (c2w0 rhog(k) + c2w1 rhog(k-1))
      double b_gh = -b_rgsh * rgsh * rgh;
      XBown(A_gam2h, ck, b_rgsh * rgh);
      b_rw = fma(b_kinv * rw, rden, b_rw);
      const double b_den = -b_kinv * kinv * rden;
      b_rhog = fma(b_den, c2w0, b_rhog);
      YBadd(YS_RHOG, c - G, b_den * c2w1);
      const double b_c2w0 = b_den * rhog, b_c2w1 = b_den * rhogm;
      b_gh += b_c2w0 * (afact[k] * rgsr) + b_c2w1 * (bfact[k] * rgsm);
      b_gs = fma(-(b_c2w0 * c2w0), rgsr, b_gs);
      XBadd(A_gsgam2, ck - G, -b_c2w1 * c2w1 * rgsm);
      XBown(A_gsgam2h, ck, b_gh);
      XBown(A_rhogw, ck, b_rw);
    }
    // kinh = 0.5 (rvx^2 + rvy^2 + rvz^2) / rhog
    const double b_sq = b_kinh * rrhog;
    b_rhog = fma(-(b_kinh * kinh), rrhog, b_rhog);
    XBown(A_rhogvx, ck, b_sq * rvx);
    XBown(A_rhogvy, ck, b_sq * rvy);
    XBown(A_rhogvz, ck, b_sq * rvz);
    // vi, vj
    XBown(A_vx, ck, b_vi * ix + b_vj * jx);
    XBown(A_vy, ck, b_vi * iy + b_vj * jy);
    XBown(A_vz, ck, b_vi * iz + b_vj * jz);
    XBadd(A_ix, cc, b_vi * vx);
    XBadd(A_iy, cc, b_vi * vy);
    XBadd(A_iz, cc, b_vi * vz);
    XBadd(A_jx, cc, b_vj * vx);
    XBadd(A_jy, cc, b_vj * vy);
    XBadd(A_jz, cc, b_vj * vz);
    // rgs = gam2 / gsgam2
    XBown(A_gam2, ck, b_rgs * rgsr);
    b_gs = fma(-(b_rgs * rgs), rgsr, b_gs);
    XBadd(A_gsgam2, ck, b_gs);
    YBadd(YS_RHOG, c, b_rhog);
  }
}

// Adjoint of S3, hand-written.  S3 is linear in the fluxes and tendencies, so
// the adjoints of the divergences at a level follow from that level's output
// adjoints alone; every cell rebuilds them for itself and its neighbours and
// gathers the adjoint of each of its 8 ntr fluxes (no atomics; written, not
// added: S3 is their only reader).  The other input adjoints are the cell's
// own, added where they live; the unit vectors, shared by a column, atomically.
struct S3Bar {
  double dq[MAX_TR], drhoe, drhophi, dkinh, du, dv, dkinv, dw;
};
__device__ __forceinline__ S3Bar s3_bars(const StageIO& io, int l, int k, int g) {
  const size_t c = io.L.f(l, k, g), NC = io.NC;
  const double B_rhog = io.WB[W_RHOG_N * NC + c], B_rhoge = io.WB[W_RHOGE_N * NC + c];
  const double B_rvx = io.WB[W_RVX_N * NC + c] + io.SB[SF_RVX * NC + c];
  const double B_rvy = io.WB[W_RVY_N * NC + c] + io.SB[SF_RVY * NC + c];
  const double B_rvz = io.WB[W_RVZ_N * NC + c] + io.SB[SF_RVZ * NC + c];
  const double B_rw = io.WB[W_RW_N * NC + c] + io.SB[SF_RW * NC + c];
  const size_t ic = io.L.c(l, g);
  const double z = io.x.a[A_z][c];
  S3Bar b;
  for (int t = 0; t < io.P.ntr; ++t)
    b.dq[t] = io.WB[(W_RQ_N + sed_tracer(t, io.P.ntr).nq) * NC + c] + B_rhog - B_rhoge * GRAV * z;
  b.drhoe = B_rhoge;
  b.drhophi = B_rhoge;
  b.dkinh = io.WB[W_KINH_N * NC + c];
  b.dkinv = io.WB[W_KINV_N * NC + c];
  b.du = B_rvx * io.x.a[A_ix][ic] + B_rvy * io.x.a[A_iy][ic] + B_rvz * io.x.a[A_iz][ic];
  b.dv = B_rvx * io.x.a[A_jx][ic] + B_rvy * io.x.a[A_jy][ic] + B_rvz * io.x.a[A_jz][ic];
  b.dw = B_rw;
  return b;
}
// adjoint of the divergence d_tf (full f < 6, half 6..7) at a level, from its S3Bar
__device__ __forceinline__ double s3_bd(const S3Bar& b, int t, int f) {
  switch (f) {
    case 0: return -b.dq[t];
    case 1: return -b.drhoe;
    case 2: return -b.drhophi;
    case 3: return -b.dkinh;
    case 4: return -b.du;
    case 5: return -b.dv;
    case 6: return -b.dkinv;
    default: return -b.dw;
  }
}

__global__ void __launch_bounds__(STAGE_THREADS) adj_s3_hw_kernel(StageIO io) {
  const Problem& P = io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const double* rdgz = P.grid + GF_RDGZ * K;
  const double* rdgzh = P.grid + GF_RDGZH * K;
  const double* SC = io.SB + (size_t)NSF * io.NC;
  const size_t ncol = (size_t)io.L.lall * io.L.G;
  const double dt = P.dt;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < io.NC; c += (size_t)gridDim.x * blockDim.x) {
    int g, k, l;
    io.L.split(c, l, k, g);
    const bool in_k = (k >= kmin && k <= kmax), in_km = (k - 1 >= kmin && k - 1 <= kmax);
    const bool hk = (k >= kmin + 1 && k <= kmax), hkp = (k + 1 >= kmin + 1 && k + 1 <= kmax);
    const S3Bar b0 = s3_bars(io, l, k, g);
    S3Bar bm{}, bp{};
    if (in_km) bm = s3_bars(io, l, k - 1, g);
    if (hkp) bp = s3_bars(io, l, k + 1, g);
    // flux adjoints
    const int ntr = P.ntr;
    for (int t = 0; t < ntr; ++t) {
      for (int f = 0; f < 6; ++f) {
        double bF = 0.0;
        if (in_km) bF += s3_bd(bm, t, f) * rdgz[k - 1];
        if (in_k) bF -= s3_bd(b0, t, f) * rdgz[k];
        io.WB[(W_F + 8 * t + f) * io.NC + c] = bF;
      }
      for (int f = 6; f < 8; ++f) {
        double bF = 0.0;
        if (hk) bF += s3_bd(b0, t, f) * rdgzh[k];
        if (hkp) bF -= s3_bd(bp, t, f) * rdgzh[k + 1];
        io.WB[(W_F + 8 * t + f) * io.NC + c] = bF;
      }
    }
    // GPREC = 0 + (-F_QR,q(k)) / dt at interior levels; the surface outputs at kmin
    if (in_k) io.WB[(W_F + 0) * io.NC + c] -= io.SB[SF_GPREC * io.NC + c] / dt;
    if (k == kmin) {
      const size_t ic = io.L.c(l, g);
      const double bp0 = SC[SC_PRECIP0 * ncol + ic], bp1 = SC[SC_PRECIP1 * ncol + ic];
      const double blh = SC[SC_LH * ncol + ic], bre = SC[SC_RHOE * ncol + ic];
      const double bph = SC[SC_RHOPHI * ncol + ic], bkn = SC[SC_RHOKIN * ncol + ic];
      double* F = io.WB + (size_t)W_F * io.NC + c;
      F[(8 * 0 + 0) * io.NC] -= bp0 / dt;
      for (int t = 1; t < ntr; ++t) F[(8 * t + 0) * io.NC] += -bp1 / dt + blh * LHF0 / dt;
      for (int t = 0; t < ntr; ++t) {
        F[(8 * t + 1) * io.NC] -= bre / dt;
        F[(8 * t + 2) * io.NC] -= bph / dt;
        F[(8 * t + 3) * io.NC] -= bkn / dt;
      }
    }
    // the cell's own inputs
    const size_t NC = io.NC;
    const double B_rhog = io.WB[W_RHOG_N * NC + c], B_rhoge = io.WB[W_RHOGE_N * NC + c];
    const double B_rvx = io.WB[W_RVX_N * NC + c] + io.SB[SF_RVX * NC + c];
    const double B_rvy = io.WB[W_RVY_N * NC + c] + io.SB[SF_RVY * NC + c];
    const double B_rvz = io.WB[W_RVZ_N * NC + c] + io.SB[SF_RVZ * NC + c];
    const double B_rw = io.WB[W_RW_N * NC + c] + io.SB[SF_RW * NC + c];
    if (in_k) {
      io.YB[YS_RHOG * NC + c] += B_rhog;
      io.YB[YS_RHOGE * NC + c] += B_rhoge;
      for (int n = 0; n < 6; ++n) io.YB[(YS_RHOGQ + n) * NC + c] += io.WB[(W_RQ_N + n) * NC + c];
    } else {
      io.xb.a[A_rhog][c] += B_rhog;
      io.xb.a[A_rhoge][c] += B_rhoge;
      for (int n = 0; n < 6; ++n) io.xb.a[A_rhogq][io.L.t(l, n, k, g)] += io.WB[(W_RQ_N + n) * NC + c];
    }
    io.xb.a[A_rhogvx][c] += B_rvx;
    io.xb.a[A_rhogvy][c] += B_rvy;
    io.xb.a[A_rhogvz][c] += B_rvz;
    io.xb.a[A_rhogw][c] += B_rw;
    io.WB[W_KINH * NC + c] = io.WB[W_KINH_N * NC + c];
    io.WB[W_KINV * NC + c] = io.WB[W_KINV_N * NC + c];
    if (in_k) {
      // the tendencies at this level (forward values) for the products with z and the unit vectors
      const double* Fw = io.W + (size_t)W_F * NC + c;
      double dqsum = 0.0, du = 0.0, dv = 0.0;
      for (int t = 0; t < ntr; ++t) {
        dqsum -= (Fw[(8 * t + 0) * NC + io.L.G] - Fw[(8 * t + 0) * NC]) * rdgz[k];
        du = du - (Fw[(8 * t + 4) * NC + io.L.G] - Fw[(8 * t + 4) * NC]) * rdgz[k];
        dv = dv - (Fw[(8 * t + 5) * NC + io.L.G] - Fw[(8 * t + 5) * NC]) * rdgz[k];
      }
      const double bz = -B_rhoge * GRAV * dqsum;
      io.xb.a[A_z][c] += bz;
      const size_t ic = io.L.c(l, g);
      atomicAdd(&io.xb.a[A_ix][ic], B_rvx * du);
      atomicAdd(&io.xb.a[A_iy][ic], B_rvy * du);
      atomicAdd(&io.xb.a[A_iz][ic], B_rvz * du);
      atomicAdd(&io.xb.a[A_jx][ic], B_rvx * dv);
      atomicAdd(&io.xb.a[A_jy][ic], B_rvy * dv);
      atomicAdd(&io.xb.a[A_jz][ic], B_rvz * dv);
    }
  }
}

// Adjoint of S2, recorded on a tape (adjoint mode 1): a work item per cell and flux.
__global__ void __launch_bounds__(STAGE_THREADS) adj_s2_kernel(StageIO io, TapeMem tm) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  __syncthreads();
  tape_bind_s(tm);
  LeafLog lg;
  const size_t n = io.NC * 8 * io.P.ntr;
  for (size_t w = tape().slot; w < n; w += tape().nslot) {
    const size_t c = w % io.NC;
    const int j = (int)(w / io.NC);
    const double gF = io.WB[(W_F + j) * io.NC + c];
    if (gF == 0.0) continue;
    int g, k, l;
    io.L.split(c, l, k, g);
    tape_begin(lg);
    const In<RVar> in{io, l, g, &lg};
    const RVar F = stage2<RVar>(in, grid, k, j);
    if (stage_overflow(io, lg, k, g, l)) continue;
    tape_clear_adj();
    seed(F, gF);
    tape_reverse();
    scatter(io, lg);
  }
}

// Adjoint of S2, hand-written: one thread per cell and tracer, for the eight
// fluxes of the tracer.  A flux is acc = sum_k2 src(k2) c(k2) + src(kc) zdis'
// where |acc| >= EPS and 0 below; the stored flux tells which (acc is never 0
// where it is kept).  The departure distances' adjoints of this cell are only
// written here; the sources' go to the levels the integral spans, by atomics.
__global__ void __launch_bounds__(STAGE_THREADS) adj_s2_hw_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int i = threadIdx.x; i < GF_COUNT * io.P.kall; i += blockDim.x) grid[i] = io.P.grid[i];
  __syncthreads();
  const Problem& P = io.P;
  const int K = P.kall, kmin = P.kmin, kmax = P.kmax;
  const size_t NC = io.NC, G = io.L.G;
  const int ntr = P.ntr;
  const size_t n = NC * ntr;
  for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < n; w += (size_t)gridDim.x * blockDim.x) {
    const size_t c = w % NC;
    const int t = (int)(w / NC);
    const int k = (int)((c / G) % K), l = (int)(c / (G * K));
    if (k < kmin || k > kmax) continue;
    const int* bmn = io.bnd + ((size_t)l * 2 + 0) * 2 * MAX_TR * K;
    const int* bmx = io.bnd + ((size_t)l * 2 + 1) * 2 * MAX_TR * K;
    for (int half = 0; half < 2; ++half) {
      const int mkmin = half ? kmin + 1 : kmin;
      if (k < mkmin) continue;
      const int f0 = half ? 6 : 0, f1 = half ? 8 : 6;
      bool any = false;
      for (int f = f0; f < f1; ++f)
        any = any || (io.WB[(W_F + 8 * t + f) * NC + c] != 0.0 && io.W[(W_F + 8 * t + f) * NC + c] != 0.0);
      if (!any) continue;
      const int r = half ? ntr + t : t;
      const int lo = bmn[r * K + k];
      const int hi = bmx[t * K + k];
      const double* zh = grid + (half ? GF_GZSHIFT : GF_GZH) * K;
      const double* dz = grid + (half ? GF_DGZH : GF_DGZ) * K;
      const double zv = io.W[(W_ZDIS + r) * NC + c];
      const int kc = departure_cell_t(zh, k, zv, lo, bmx[r * K + k], mkmin, kmax);
      const bool span = !(lo == k && hi == k);
      double zd = zv;
      if (span && hi != kc) zd = zd - (hi > kc ? dz[hi] : -dz[hi]);
      double b_z = 0.0;
      for (int f = f0; f < f1; ++f) {
        const double gF = io.WB[(W_F + 8 * t + f) * NC + c];
        if (gF == 0.0 || io.W[(W_F + 8 * t + f) * NC + c] == 0.0) continue;
        const int src = W_RHOF + 8 * t + f;
        double* bs = io.WB + (size_t)src * NC + (c - (size_t)k * G);   // level 0 of this column
        if (span)
          for (int k2 = lo; k2 <= hi; ++k2) {
            if (k2 == kc) continue;
            atomicAdd(bs + (size_t)k2 * G, gF * (k2 > kc ? dz[k2] : -dz[k2]));
          }
        if (zd != 0.0) atomicAdd(bs + (size_t)kc * G, gF * zd);
        b_z = fma(gF, io.W[(size_t)src * NC + (c - (size_t)k * G) + (size_t)kc * G], b_z);
      }
      io.WB[(W_ZDIS + r) * NC + c] += b_z;
    }
  }
}

// Adjoint of S1, recorded on a tape (adjoint mode 1): seeds from S2's and S3's adjoints (WB).
__global__ void __launch_bounds__(STAGE_THREADS) adj_s1_kernel(StageIO io, TapeMem tm) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  __syncthreads();
  tape_bind_s(tm);
  LeafLog lg;
  for (size_t c = tape().slot; c < io.NC; c += tape().nslot) {
    int g, k, l;
    io.L.split(c, l, k, g);
    tape_begin(lg);
    const In<RVar> in{io, l, g, &lg};
    RVar o[W_F];
    stage1<RVar>(in, grid, k, [&](int f, const RVar& v) { o[f] = v; });
    if (stage_overflow(io, lg, k, g, l)) continue;
    tape_clear_adj();
    for (int f = 0; f < W_F; ++f) seed(o[f], io.WB[f * io.NC + c]);
    tape_reverse();
    scatter(io, lg);
  }
}

// Copies the caller's output adjoints of the column phase into the seed
// buffer and clears them there (input adjoints are then added in place).
__global__ void adj_seed_kernel(StageIO io) {
  const LayS& L = io.L;
  double* SB = const_cast<double*>(io.SB);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < io.NC; c += (size_t)gridDim.x * blockDim.x) {
    int g, k, l;
    L.split(c, l, k, g);
    auto take = [&](int f, int a, size_t i) {
      SB[f * io.NC + c] = io.xb.a[a][i];
      io.xb.a[a][i] = 0.0;
    };
    take(SF_RHOG, A_rhog, c);
    take(SF_RHOGE, A_rhoge, c);
    take(SF_RVX, A_rhogvx, c);
    take(SF_RVY, A_rhogvy, c);
    take(SF_RVZ, A_rhogvz, c);
    take(SF_RW, A_rhogw, c);
    take(SF_RHO, A_rho, c);
    take(SF_TEM, A_tem, c);
    take(SF_PRE, A_pre, c);
    take(SF_QD, A_qd, c);
    take(SF_GPREC, A_GPREC, c);
    for (int n = 0; n < 6; ++n) {
      take(SF_RQ + n, A_rhogq, L.t(l, n, k, g));
      take(SF_Q + n, A_q, L.t(l, n, k, g));
    }
    io.xb.a[A_re_solid][c] = 0.0;
    io.xb.a[A_GDCLW][c] = 0.0;
    io.xb.a[A_GDCFRC][c] = 0.0;
    // outputs of the cell phase (interior levels): their adjoints go to YB
    const bool interior = (k >= io.P.kmin && k <= io.P.kmax);
    io.YB[YS_RE * io.NC + c] = interior ? io.xb.a[A_re_liquid][c] : 0.0;
    io.YB[YS_RECLD * io.NC + c] = interior ? io.xb.a[A_re_cld][c] : 0.0;
    io.xb.a[A_re_liquid][c] = 0.0;
    io.xb.a[A_re_cld][c] = 0.0;
    if (k == io.P.kmax) {
      // rwtop = sw rctop + (1 - sw) UNDEF with sw from tctop (TagUpdateCLD)
      const size_t ic = L.c(l, g);
      const double sw = (0.5 + copysign(0.5, io.Y[YS_TCTOP * io.NC + c] - TEM00));
      io.YB[YS_RCTOP * io.NC + c] = io.xb.a[A_rctop][ic] + sw * io.xb.a[A_rwtop][ic];
      io.YB[YS_TCTOP * io.NC + c] = io.xb.a[A_tctop][ic];
    }
    if (k == 0) {
      const size_t ncol = (size_t)L.lall * L.G;
      double* SC = SB + (size_t)NSF * io.NC;
      const size_t ic = L.c(l, g);
      auto takec = [&](int f, int a, size_t i) {
        SC[f * ncol + ic] = io.xb.a[a][i];
        io.xb.a[a][i] = 0.0;
      };
      takec(SC_PRECIP0, A_precip, L.p(0, l, g));
      takec(SC_PRECIP1, A_precip, L.p(1, l, g));
      takec(SC_LH, A_precip_lh_heat, ic);
      takec(SC_RHOE, A_precip_rhoe, ic);
      takec(SC_RHOPHI, A_precip_rhophi, ic);
      takec(SC_RHOKIN, A_precip_rhokin, ic);
      io.xb.a[A_ISO1][L.p(0, l, g)] = 0.0;
      io.xb.a[A_ISO1][L.p(1, l, g)] = 0.0;
      io.xb.a[A_ISO2][L.p(0, l, g)] = 0.0;
      io.xb.a[A_ISO2][L.p(1, l, g)] = 0.0;
    }
  }
}

// Clears the caller's adjoints of the cloud-top outputs (read by the seed
// kernel at the top interior level).
__global__ void adj_seed_columns_kernel(StageIO io) {
  const size_t ncol = (size_t)io.L.lall * io.L.G;
  for (size_t ic = (size_t)blockIdx.x * blockDim.x + threadIdx.x; ic < ncol; ic += (size_t)gridDim.x * blockDim.x) {
    io.xb.a[A_rctop][ic] = 0.0;
    io.xb.a[A_rwtop][ic] = 0.0;
    io.xb.a[A_tctop][ic] = 0.0;
  }
}

// The cell phase's adjoint, hand-written (nsw6_cell_adjoint.cuh): one thread
// per interior cell; output adjoints from YB, input adjoints added to xb (each
// cell owns its entries here), the parameters' adjoint reduced per block.
// R = double: the FP64 cell physics (table-driven exp / log / pow); R = float:
// the mixed-precision one (FP32 rates with the CUDA FP32 math functions, FP64
// budgets), as the step's cell kernel evaluates them.
template <class R>
struct CellMath;
template <>
struct CellMath<double> {
  using M = FastMath;
  __device__ static M make(const double* tab) {
    return FastMath{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  }
};
template <>
struct CellMath<float> {
  using M = FloatMath;
  __device__ static M make(const double*) { return FloatMath{}; }
};

// The cell phase's forward for the adjoint: the outputs Y of every interior
// cell and the checkpoint of its costly forward values (CELL_CK_SLOTS doubles,
// slot-major over the cells), both from the hand-written forward.  check: also
// evaluate nsw6_cell and report a cell whose outputs differ in any bit
// (status ERR_ADJ_CHECK, iters = the first output field that differs).
constexpr int ERR_ADJ_CHECK = 7;
template <class R>
__global__ void __launch_bounds__(128) adj_cell_save_kernel(Problem P, ConstsT<R> C, ArgPtrs x, double* Y, double* ck,
                                                            int check) {
  __shared__ double tab[FM_TABLE_DOUBLES];
  if constexpr (sizeof(R) == sizeof(double)) {
    for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = P.fmtab[c];
    __syncthreads();
  }
  const auto fm = CellMath<R>::make(tab);
  const LayS L{P.kall, P.gall, P.lall, P.prec_ld};
  const size_t NC = (size_t)P.lall * P.kall * P.gall;
  const int nint = P.kmax - P.kmin + 1;
  const FastDiv dg = FastDiv::make((unsigned)P.gall), dn = FastDiv::make((unsigned)nint);
  const long long ncell = (long long)P.lall * nint * P.gall;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const unsigned ci = (unsigned)c, q = dg.div(ci), q2 = dn.div(q);   // ncell < 2^32
    const int g = (int)(ci - q * (unsigned)P.gall);
    const int k = P.kmin + (int)(q - q2 * (unsigned)nint);
    const int l = (int)q2;
    const size_t i = L.f(l, k, g);
    CellIn in;
    in.rhog = x.a[A_rhog][i];
    in.tem = x.a[A_tem][i];
    in.gsgam2 = x.a[A_gsgam2][i];
    in.q0 = x.a[A_q][L.t(l, 0, k, g)];
    for (int n = 0; n < 6; ++n) in.rhogq[n] = x.a[A_rhogq][L.t(l, n, k, g)];
    CellOut o;
    CellBar ob{};
    CellInBar ib{};
    nsw6_cell_adjoint<CA_SAVE>(C, fm, P.dt, P.rdt, in, ob, ib, nullptr, CellCk{ck, (size_t)ncell, (size_t)c}, &o);
    double y[ADJ_Y_FIELDS];
    y[YS_RHOG] = o.rhog;
    y[YS_RHOGE] = o.rhoge;
    y[YS_TEM] = o.tem;
    for (int n = 0; n < 6; ++n) y[YS_RHOGQ + n] = o.rhogq[n];
    for (int n = 1; n < 6; ++n) y[YS_Q + n - 1] = o.q[n];
    y[YS_VT + 0] = o.Vtr;
    y[YS_VT + 1] = o.Vts;
    y[YS_VT + 2] = o.Vtg;
    y[YS_VT + 3] = 0.0;   // QI does not sediment in this (switch-free) cell phase
    y[YS_RE] = o.rceff;
    y[YS_RECLD] = o.rceff_cld;
    y[YS_RCTOP] = o.rctop;
    y[YS_TCTOP] = o.tctop;
    for (int f = 0; f < ADJ_Y_FIELDS; ++f) Y[f * NC + i] = y[f];
    if (check) {
      CellOut r;
      nsw6_cell<typename CellMath<R>::M, R, double>(C, fm, P.dt, P.rdt, in, r);
      double z[ADJ_Y_FIELDS];
      z[YS_RHOG] = r.rhog;
      z[YS_RHOGE] = r.rhoge;
      z[YS_TEM] = r.tem;
      for (int n = 0; n < 6; ++n) z[YS_RHOGQ + n] = r.rhogq[n];
      for (int n = 1; n < 6; ++n) z[YS_Q + n - 1] = r.q[n];
      z[YS_VT + 0] = r.Vtr;
      z[YS_VT + 1] = r.Vts;
      z[YS_VT + 2] = r.Vtg;
      z[YS_VT + 3] = 0.0;
      z[YS_RE] = r.rceff;
      z[YS_RECLD] = r.rceff_cld;
      z[YS_RCTOP] = r.rctop;
      z[YS_TCTOP] = r.tctop;
      for (int f = 0; f < ADJ_Y_FIELDS; ++f)
        if (__double_as_longlong(y[f]) != __double_as_longlong(z[f])) {
          record_err(P.status, ERR_ADJ_CHECK, k, g, l, f);
          break;
        }
    }
  }
}

// The cell phase's adjoint, hand-written, from the checkpoint ck of
// adj_cell_save_kernel.
template <class R>
__global__ void __launch_bounds__(128) adj_cell_hw_kernel(Problem P, ConstsT<R> C, ArgPtrs x, ArgPtrs xb,
                                                          const double* YB, double* pbar, double* ck) {
  __shared__ double tab[FM_TABLE_DOUBLES];
  __shared__ double red[7][128];
  if constexpr (sizeof(R) == sizeof(double))
    for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = P.fmtab[c];
  __syncthreads();
  const auto fm = CellMath<R>::make(tab);
  const LayS L{P.kall, P.gall, P.lall, P.prec_ld};
  const size_t NC = (size_t)P.lall * P.kall * P.gall;
  const int nint = P.kmax - P.kmin + 1;
  const FastDiv dg = FastDiv::make((unsigned)P.gall), dn = FastDiv::make((unsigned)nint);
  const long long ncell = (long long)P.lall * nint * P.gall;
  double pacc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const unsigned ci = (unsigned)c, q = dg.div(ci), q2 = dn.div(q);   // ncell < 2^32
    const int g = (int)(ci - q * (unsigned)P.gall);
    const int k = P.kmin + (int)(q - q2 * (unsigned)nint);
    const int l = (int)q2;
    const size_t i = L.f(l, k, g);
    CellIn in;
    in.rhog = x.a[A_rhog][i];
    in.tem = x.a[A_tem][i];
    in.gsgam2 = x.a[A_gsgam2][i];
    in.q0 = x.a[A_q][L.t(l, 0, k, g)];
    for (int n = 0; n < 6; ++n) in.rhogq[n] = x.a[A_rhogq][L.t(l, n, k, g)];
    CellBar ob;
    ob.rhog = YB[YS_RHOG * NC + i];
    ob.rhoge = YB[YS_RHOGE * NC + i];
    ob.tem = YB[YS_TEM * NC + i];
    for (int n = 0; n < 6; ++n) ob.rhogq[n] = YB[(YS_RHOGQ + n) * NC + i];
    ob.q[0] = 0.0;
    for (int n = 1; n < 6; ++n) ob.q[n] = YB[(YS_Q + n - 1) * NC + i];
    ob.Vtr = YB[(YS_VT + 0) * NC + i];
    ob.Vts = YB[(YS_VT + 1) * NC + i];
    ob.Vtg = YB[(YS_VT + 2) * NC + i];
    ob.rceff = YB[YS_RE * NC + i];
    ob.rceff_cld = YB[YS_RECLD * NC + i];
    ob.rctop = k == P.kmax ? YB[YS_RCTOP * NC + i] : 0.0;
    ob.tctop = k == P.kmax ? YB[YS_TCTOP * NC + i] : 0.0;
    CellInBar ib{};
    nsw6_cell_adjoint<CA_LOAD>(C, fm, P.dt, P.rdt, in, ob, ib, pacc, CellCk{ck, (size_t)ncell, (size_t)c});
    xb.a[A_rhog][i] += ib.rhog;
    xb.a[A_tem][i] += ib.tem;
    xb.a[A_gsgam2][i] += ib.gsgam2;
    xb.a[A_q][L.t(l, 0, k, g)] += ib.q0;
    for (int n = 0; n < 6; ++n) xb.a[A_rhogq][L.t(l, n, k, g)] += ib.rhogq[n];
  }
  for (int j = 0; j < 7; ++j) red[j][threadIdx.x] = pacc[j];
  __syncthreads();
  if (threadIdx.x < 7) {
    double sum = 0.0;
    for (int j = 0; j < (int)blockDim.x; ++j) sum += red[threadIdx.x][j];
    atomicAdd(&pbar[threadIdx.x], sum);
  }
}

// ------------------------------------------------------------------ tangent-linear step in stages
// The same stages in forward mode (T = Dual): every cell of every column in
// parallel.  StageIO's adjoint arrays hold the tangents here: xb the step's
// argument tangents (read as inputs, written as outputs), YB the cell
// outputs' tangents, WB the work fields' tangents.  The values of the work
// fields and the flux bounds come from the forward kernels above.  The last
// two stages also write the step's output values: the stage functions make
// the production kernels' operations on the same values, so they are those
// kernels' outputs bit for bit (tested against the step).
template <>
struct In<Dual> {
  const StageIO& io;
  int l, g;
  __device__ Dual w(int f, int kk) const {
    const size_t i = f * io.NC + io.L.f(l, kk, g);
    return Dual(io.W[i], io.WB[i]);
  }
  __device__ Dual y(int f, int kk) const {
    const size_t i = f * io.NC + io.L.f(l, kk, g);
    return Dual(io.Y[i], io.YB[i]);
  }
  __device__ Dual x(int a, size_t i) const { return Dual(io.x.a[a][i], io.xb.a[a][i]); }
};

// Cell phase in forward mode: the FP64 cell physics over Dual (parameter
// tangents through the folded constants), its outputs' values into Y and
// tangents into YB.  The constants (one copy per block) sit in shared memory.
template <bool OPT>
__global__ void __launch_bounds__(128) tlm_cell_kernel(StageIO io, Consts C, const double* params,
                                                       const double* dparams) {
  __shared__ double tab[FM_TABLE_DOUBLES];
  __shared__ __align__(16) unsigned char ct_raw[sizeof(ConstsT<Dual>)];
  ConstsT<Dual>& CT = *reinterpret_cast<ConstsT<Dual>*>(ct_raw);
  const Problem& P = io.P;
  for (int c = threadIdx.x; c < FM_TABLE_DOUBLES; c += blockDim.x) tab[c] = P.fmtab[c];
  if (threadIdx.x == 0) {
    Dual p[7];
    for (int i = 0; i < 7; ++i) p[i] = Dual(params[i], dparams ? dparams[i] : 0.0);
    consts_with_params(C, p, CT);
  }
  __syncthreads();
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  const ADMath<Dual> mth{fm};
  const LayS& L = io.L;
  const size_t NC = io.NC;
  const int nint = P.kmax - P.kmin + 1;
  const FastDiv dg = FastDiv::make((unsigned)P.gall), dn = FastDiv::make((unsigned)nint);
  const long long ncell = (long long)P.lall * nint * P.gall;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const unsigned ci = (unsigned)c, q = dg.div(ci), q2 = dn.div(q);   // ncell < 2^32
    const int g = (int)(ci - q * (unsigned)P.gall);
    const int k = P.kmin + (int)(q - q2 * (unsigned)nint);
    const int l = (int)q2;
    const size_t i = L.f(l, k, g);
    const In<Dual> x{io, l, g};
    CellInT<Dual> in;
    in.rhog = x.x(A_rhog, i);
    in.tem = x.x(A_tem, i);
    in.gsgam2 = x.x(A_gsgam2, i);
    in.q0 = x.x(A_q, L.t(l, 0, k, g));
    for (int n = 0; n < 6; ++n) in.rhogq[n] = x.x(A_rhogq, L.t(l, n, k, g));
    // the CCN field (aerosol switch) is an input without a tangent
    in.unccn = Dual((OPT && io.x.a[A_unccn]) ? io.x.a[A_unccn][i] : 0.0);
    CellOutT<Dual> o;
    nsw6_cell<ADMath<Dual>, Dual, Dual, OPT>(CT, mth, P.dt, P.rdt, in, o);
    auto put = [&](int f, const Dual& v) {
      io.YB[f * NC + i] = v.d;
      const_cast<double*>(io.Y)[f * NC + i] = v.v;
    };
    put(YS_RHOG, o.rhog);
    put(YS_RHOGE, o.rhoge);
    put(YS_TEM, o.tem);
    for (int n = 0; n < 6; ++n) put(YS_RHOGQ + n, o.rhogq[n]);
    for (int n = 1; n < 6; ++n) put(YS_Q + n - 1, o.q[n]);
    put(YS_VT + 0, o.Vtr);
    put(YS_VT + 1, o.Vts);
    put(YS_VT + 2, o.Vtg);
    put(YS_VT + 3, o.Vti);
    put(YS_RE, o.rceff);
    put(YS_RECLD, o.rceff_cld);
    put(YS_RCTOP, o.rctop);
    put(YS_TCTOP, o.tctop);
  }
}

// S1 in forward mode: the work fields' tangents.
__global__ void __launch_bounds__(STAGE_THREADS) tlm_s1_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  __syncthreads();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < io.NC; c += (size_t)gridDim.x * blockDim.x) {
    int g, k, l;
    io.L.split(c, l, k, g);
    const In<Dual> in{io, l, g};
    stage1<Dual>(in, grid, k, [&](int f, const Dual& v) { io.WB[f * io.NC + c] = v.d; });
  }
}

// S2 in forward mode (a work item per cell and flux).
__global__ void __launch_bounds__(STAGE_THREADS) tlm_s2_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  __syncthreads();
  const int nj = 8 * io.P.ntr;
  for (int j = 0; j < nj; ++j)
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < io.NC; c += (size_t)gridDim.x * blockDim.x) {
      int g, k, l;
      io.L.split(c, l, k, g);
      const In<Dual> in{io, l, g};
      io.WB[(W_F + j) * io.NC + c] = stage2<Dual>(in, grid, k, j).d;
    }
}

// S3 in forward mode: work-field tangents, and the values and tangents of the
// step's momentum, GPREC and surface outputs.
__global__ void __launch_bounds__(STAGE_THREADS) tlm_s3_kernel(StageIO io) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  for (int c = threadIdx.x; c < GF_COUNT * io.P.kall; c += blockDim.x) grid[c] = io.P.grid[c];
  __syncthreads();
  const LayS& L = io.L;
  double* const* x = io.x.a;
  double* const* dx = io.xb.a;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < io.NC; c += (size_t)gridDim.x * blockDim.x) {
    int g, k, l;
    L.split(c, l, k, g);
    const In<Dual> in{io, l, g};
    const size_t ic = L.c(l, g);
    auto out = [&](int a, size_t i, const Dual& v) {
      x[a][i] = v.v;
      dx[a][i] = v.d;
    };
    // GPREC: from the surface-ward flux at the interior levels, 0 elsewhere
    if (k < io.P.kmin || k > io.P.kmax) out(A_GPREC, c, Dual(0.0));
    stage3<Dual>(
        in, grid, k, [&](int f, const Dual& v) { io.WB[f * io.NC + c] = v.d; },
        [&](int f, const Dual& v) {
          if (io.kin2kin && f != SF_GPREC) return;   // S4 gives the momenta
          const int a = f == SF_RVX ? A_rhogvx : f == SF_RVY ? A_rhogvy : f == SF_RVZ ? A_rhogvz
                      : f == SF_RW ? A_rhogw : A_GPREC;
          out(a, c, v);
        },
        [&](int f, const Dual& v) {
          switch (f) {
            case SC_PRECIP0: out(A_precip, L.p(0, l, g), v); break;
            case SC_PRECIP1: out(A_precip, L.p(1, l, g), v); break;
            case SC_LH: out(A_precip_lh_heat, ic, v); break;
            case SC_RHOE: out(A_precip_rhoe, ic, v); break;
            case SC_RHOPHI: out(A_precip_rhophi, ic, v); break;
            default: out(A_precip_rhokin, ic, v); break;
          }
        });
  }
}

// S4 in forward mode: the values and tangents of the step's state outputs, of
// the outputs the cell phase gives directly (effective radii, cloud top) and
// of those the step sets to constants (the mp_driver epilogue,
// mod_mp_driver.cpp:555-612; zero tangents).
__global__ void __launch_bounds__(STAGE_THREADS) tlm_s4_kernel(StageIO io, Consts C) {
  __shared__ double grid[GF_COUNT * MAX_KALL];
  __shared__ double tab[FM_TABLE_DOUBLES];
  stage_smem(io.P, grid, tab);
  const FastMath fm{tab, tab + FM_EXP_N, tab + 2 * FM_EXP_N, tab + 2 * FM_EXP_N + FM_LOG_N};
  const LayS& L = io.L;
  const size_t NC = io.NC;
  double* const* x = io.x.a;
  double* const* dx = io.xb.a;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < NC; c += (size_t)gridDim.x * blockDim.x) {
    int g, k, l;
    L.split(c, l, k, g);
    const In<Dual> in{io, l, g};
    auto out = [&](int a, size_t i, const Dual& v) {
      x[a][i] = v.v;
      dx[a][i] = v.d;
    };
    auto y = [&](int f) { return Dual(io.Y[f * NC + c], io.YB[f * NC + c]); };
    int it = 0;
    const int rc = stage4<Dual>(in, C, grid, fm, k, [&](int f, const Dual& v) {
      if (f == SF_RHOG) out(A_rhog, c, v);
      else if (f == SF_RHOGE) out(A_rhoge, c, v);
      else if (f == SF_RHO) out(A_rho, c, v);
      else if (f == SF_TEM) out(A_tem, c, v);
      else if (f == SF_PRE) out(A_pre, c, v);
      else if (f == SF_QD) out(A_qd, c, v);
      else if (f >= SF_RQ && f < SF_RQ + 6) out(A_rhogq, L.t(l, f - SF_RQ, k, g), v);
      else if (f >= SF_Q && f < SF_Q + 6) out(A_q, L.t(l, f - SF_Q, k, g), v);
      else if (f == SF_RVX) out(A_rhogvx, c, v);
      else if (f == SF_RVY) out(A_rhogvy, c, v);
      else if (f == SF_RVZ) out(A_rhogvz, c, v);
      else if (f == SF_RW) out(A_rhogw, c, v);
    }, &it);
    if (rc) record_err(io.P.status, rc, k, g, l, it);
    const bool interior = (k >= io.P.kmin && k <= io.P.kmax);
    out(A_re_liquid, c, interior ? y(YS_RE) : Dual(0.0));
    out(A_re_cld, c, interior ? y(YS_RECLD) : Dual(0.0));
    out(A_re_solid, c, Dual(20.0E-6));
    out(A_GDCLW, c, Dual(0.0));
    out(A_GDCFRC, c, Dual(0.0));
    if (k == io.P.kmax) {
      // cloud top (TagUpdateCLD): rwtop = sw rctop + (1 - sw) UNDEF, sw from tctop
      const size_t ic = L.c(l, g);
      const Dual rct = y(YS_RCTOP), tct = y(YS_TCTOP);
      const double sw = (0.5 + copysign(0.5, tct.v - TEM00));
      out(A_rctop, ic, rct);
      out(A_tctop, ic, tct);
      x[A_rwtop][ic] = (sw)*rct.v + (1.0 - sw) * UNDEF;
      dx[A_rwtop][ic] = sw * rct.d;
    }
    if (k == 0) {
      out(A_ISO1, L.p(0, l, g), Dual(0.0));
      out(A_ISO1, L.p(1, l, g), Dual(0.0));
      out(A_ISO2, L.p(0, l, g), Dual(0.0));
      out(A_ISO2, L.p(1, l, g), Dual(0.0));
    }
  }
}

}  // namespace

// ------------------------------------------------------------------ launchers
size_t adj_stage_work_doubles(int lall, int kall, int gall) {
  const size_t NC = (size_t)lall * kall * gall;
  return 2 * (size_t)NWF * NC + (size_t)NSF * NC + (size_t)NSC * lall * gall;
}
size_t adj_stage_bound_ints(int lall, int kall) { return (size_t)lall * 2 * 2 * MAX_TR * kall; }
int adj_stage_tape_cap() { return 512; }
int adj_stage_slots() { return 152 * 4 * STAGE_THREADS; }

// mixed: the cell phase of the mixed-precision step (FP32 rates).
cudaError_t launch_adj_cell_hw(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& xb, const double* YB,
                               double* pbar, double* ck, int mixed, cudaStream_t stream) {
  if (mixed)
    adj_cell_hw_kernel<float><<<152 * 2, 128, 0, stream>>>(P, consts_to_float(C), x, xb, YB, pbar, ck);
  else
    adj_cell_hw_kernel<double><<<152 * 2, 128, 0, stream>>>(P, C, x, xb, YB, pbar, ck);
  return cudaGetLastError();
}

// The tangent-linear step in stages: the cell phase in forward mode (Y and
// its tangents), the column phase's forward values and flux bounds, then its
// stages in forward mode writing the step's outputs into x and their tangents
// into dx.  Y holds 2 x ADJ_Y_FIELDS fields (values, tangents); work as for
// the adjoint.
cudaError_t launch_tlm_staged(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& dx,
                              const double* params, const double* dparams, double* Y, double* work, int* bnd,
                              cudaStream_t stream) {
  StageIO io;
  io.P = P;
  io.L = LayS{P.kall, P.gall, P.lall, P.prec_ld, FastDiv::make((unsigned)P.gall), FastDiv::make((unsigned)P.kall)};
  io.NC = (size_t)P.lall * P.kall * P.gall;
  io.x = x;
  io.xb = dx;
  io.Y = Y;
  io.YB = Y + (size_t)ADJ_Y_FIELDS * io.NC;
  io.W = work;
  io.WB = work + (size_t)NWF * io.NC;
  io.SB = nullptr;
  io.bnd = bnd;
  io.kin2kin = P.opt && C.opt_kin2kin != 0.0;
  cudaError_t e;
  const size_t nkey = (size_t)P.lall * 2 * P.ntr * P.kall;
  if ((e = cudaMemsetAsync(P.zmax, 0x00, nkey * sizeof(unsigned long long), stream)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(P.zmin, 0xff, nkey * sizeof(unsigned long long), stream)) != cudaSuccess) return e;
  if (P.opt)
    tlm_cell_kernel<true><<<152 * 4, 128, 0, stream>>>(io, C, params, dparams);
  else
    tlm_cell_kernel<false><<<152 * 4, 128, 0, stream>>>(io, C, params, dparams);
  adj_s1_fwd_kernel<false><<<dim3((P.gall + STAGE_THREADS - 1) / STAGE_THREADS, P.kall, P.lall), STAGE_THREADS, 0, stream>>>(
      io);
  adj_bounds_kernel<<<(int)((nkey + 127) / 128), 128, 0, stream>>>(P, bnd);
  adj_s2_fwd_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  adj_s3_fwd_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  tlm_s1_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  tlm_s2_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  tlm_s3_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  tlm_s4_kernel<<<152 * 4, STAGE_THREADS, 0, stream>>>(io, C);
  return cudaGetLastError();
}

int adj_y_fields() { return ADJ_Y_FIELDS; }

size_t adj_cell_ck_doubles(int lall, int kall, int gall) { return (size_t)CELL_CK_SLOTS * lall * (kall - 2) * gall; }

cudaError_t launch_adj_cell_save(const Problem& P, const Consts& C, const ArgPtrs& x, double* Y, double* ck, int check,
                                 int mixed, cudaStream_t stream) {
  if (mixed)
    adj_cell_save_kernel<float><<<152 * 4, 128, 0, stream>>>(P, consts_to_float(C), x, Y, ck, check);
  else
    adj_cell_save_kernel<double><<<152 * 4, 128, 0, stream>>>(P, C, x, Y, ck, check);
  return cudaGetLastError();
}

// The column phase's adjoint: its forward S1..S3 from the state x and the cell
// phase's outputs Y (S1 also forms the region extrema of the departure
// distances in P.zmax / P.zmin, and from them the flux bounds), then the
// adjoints S4..S1 into YB (zeroed here first) and xb.  work: adj_stage_work_doubles doubles; bnd: adj_stage_bound_ints ints;
// tm: adj_stage_slots() slots of adj_stage_tape_cap() entries.
// mixed (not with recorded): the departure distances of the mixed-precision
// step (FP32), whose bounds and departure cells the stages then hold.
cudaError_t launch_adj_column_staged(const Problem& P, const Consts& C, const ArgPtrs& x, const ArgPtrs& xb,
                                     const double* Y, double* YB, int ny, double* work, int* bnd, const TapeMem& tm,
                                     int recorded, int mixed, cudaStream_t stream) {
  if (recorded && mixed) return cudaErrorInvalidValue;
  StageIO io;
  io.P = P;
  io.L = LayS{P.kall, P.gall, P.lall, P.prec_ld, FastDiv::make((unsigned)P.gall), FastDiv::make((unsigned)P.kall)};
  io.NC = (size_t)P.lall * P.kall * P.gall;
  io.x = x;
  io.xb = xb;
  io.Y = Y;
  io.YB = YB;
  io.W = work;
  io.WB = work + (size_t)NWF * io.NC;
  io.SB = work + 2 * (size_t)NWF * io.NC;
  io.bnd = bnd;
  io.kin2kin = P.opt && C.opt_kin2kin != 0.0;
  const int blocks = tm.nslot / STAGE_THREADS;
  cudaError_t e;
  if ((e = cudaMemsetAsync(io.WB, 0, sizeof(double) * NWF * io.NC, stream)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(YB, 0, sizeof(double) * ny * io.NC, stream)) != cudaSuccess) return e;
  const size_t nkey = (size_t)P.lall * 2 * P.ntr * P.kall;
  if ((e = cudaMemsetAsync(P.zmax, 0x00, nkey * sizeof(unsigned long long), stream)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(P.zmin, 0xff, nkey * sizeof(unsigned long long), stream)) != cudaSuccess) return e;
  const dim3 s1grid((P.gall + STAGE_THREADS - 1) / STAGE_THREADS, P.kall, P.lall);
  if (mixed)
    adj_s1_fwd_kernel<true><<<s1grid, STAGE_THREADS, 0, stream>>>(io);
  else
    adj_s1_fwd_kernel<false><<<s1grid, STAGE_THREADS, 0, stream>>>(io);
  adj_bounds_kernel<<<(int)((nkey + 127) / 128), 128, 0, stream>>>(P, bnd);
  adj_s2_fwd_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  adj_s3_fwd_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  adj_seed_kernel<<<152 * 4, 256, 0, stream>>>(io);
  adj_seed_columns_kernel<<<64, 256, 0, stream>>>(io);
  // S4 recorded also with the mixed-phase saturation adjustment and with
  // KIN2KIN, which the hand-written sweep does not cover
  if (recorded || (P.opt && C.opt_expice == 0.0) || io.kin2kin) {
    adj_s4_kernel<<<blocks, STAGE_THREADS, 0, stream>>>(io, C, tm);
  } else {
    // first pass: the unsaturated cells, the saturated ones listed; second: those
    if ((e = cudaMemsetAsync(P.satq, 0, sizeof(unsigned), stream)) != cudaSuccess) return e;
    adj_s4_hw_kernel<<<152 * 4, STAGE_THREADS, 0, stream>>>(io, C, 0);
    adj_s4_hw_kernel<<<152 * 4, STAGE_THREADS, 0, stream>>>(io, C, 1);
  }
  adj_s3_hw_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  if (recorded)
    adj_s2_kernel<<<blocks, STAGE_THREADS, 0, stream>>>(io, tm);
  else
    adj_s2_hw_kernel<<<152 * 8, STAGE_THREADS, 0, stream>>>(io);
  if (recorded)
    adj_s1_kernel<<<blocks, STAGE_THREADS, 0, stream>>>(io, tm);
  else if (mixed)
    adj_s1_hw_kernel<true><<<152 * 4, STAGE_THREADS, 0, stream>>>(io);
  else
    adj_s1_hw_kernel<false><<<152 * 4, STAGE_THREADS, 0, stream>>>(io);
  return cudaGetLastError();
}

}  // namespace nsw6
