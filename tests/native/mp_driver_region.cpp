// A C++ caller of the per-region drop-in mp_driver, written as the reference
// harness's call site would be (src/main.cpp:202-259 and 261-319): the
// all-regions arrays live on the device, region l's arguments are the data
// pointers of its subviews, and precip / ISO1_precip / ISO2_precip are the
// subviews (ALL, l, 0, ALL) of [2][lall][1][gall] arrays, whose rows are
// lall * gall doubles apart (nsw6_set_precip_stride).  Built with g++ against
// include/nsw6.h and the library by tests/test_gpu_native_caller.py.
//
// usage: mp_driver_region <in.bin> <out.bin>
//   in.bin:  int32 gall, kall, lall, l; float64 dt; gz[kall]; gzh[kall]; then
//            the 50 arguments in the reference order, all-regions layout
//   out.bin: the 50 arguments after the call, same layout
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "nsw6.h"

namespace {

// Shape kind of each argument, in the reference order (mod_mp_driver.h:71-124):
// 0 [k][g] field, 1 [6][k][g] tracers, 2 [2][g] precipitation, 3 [g], 4 [1][g].
const int kKind[50] = {0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 2, 2, 2, 3, 3, 3, 3, 0,
                       0, 0, 4, 4, 4, 0, 0, 0, 0, 0, 0, 0, 0, 3, 3, 3, 3, 3, 3, 0, 0, 0, 0, 0, 0};

size_t count(int kind, size_t lall, size_t kall, size_t gall) {
  switch (kind) {
    case 0: return lall * kall * gall;
    case 1: return lall * 6 * kall * gall;
    case 2: return 2 * lall * gall;
    default: return lall * gall;
  }
}

// Offset of region l's subview in an all-regions array.
size_t region_offset(int kind, size_t l, size_t kall, size_t gall) {
  switch (kind) {
    case 0: return l * kall * gall;
    case 1: return l * 6 * kall * gall;
    default: return l * gall;   // [2][lall][gall] row 0, [lall][gall], [lall][1][gall]
  }
}

bool ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
  return false;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[4];
  double dt;
  if (std::fread(hdr, sizeof(int), 4, f) != 4 || std::fread(&dt, sizeof(double), 1, f) != 1) return 2;
  const int gall = hdr[0], kall = hdr[1], lall = hdr[2], l = hdr[3];
  std::vector<double> gz(kall), gzh(kall);
  if (std::fread(gz.data(), sizeof(double), kall, f) != (size_t)kall ||
      std::fread(gzh.data(), sizeof(double), kall, f) != (size_t)kall)
    return 2;
  std::vector<std::vector<double>> host(50);
  double* dev[50] = {};
  for (int a = 0; a < 50; ++a) {
    const size_t n = count(kKind[a], lall, kall, gall);
    host[a].resize(n);
    if (std::fread(host[a].data(), sizeof(double), n, f) != n) return 2;
    if (!ok(cudaMalloc(&dev[a], n * sizeof(double)), "cudaMalloc") ||
        !ok(cudaMemcpy(dev[a], host[a].data(), n * sizeof(double), cudaMemcpyHostToDevice), "copy in"))
      return 3;
  }
  std::fclose(f);

  // region l's subviews (the data() of the reference harness's sub_* views)
  double* sub[50];
  for (int a = 0; a < 50; ++a) sub[a] = dev[a] + region_offset(kKind[a], l, kall, gall);
  double *sub_rhog = sub[0], *sub_rhogvx = sub[1], *sub_rhogvy = sub[2], *sub_rhogvz = sub[3];
  double *sub_rhogw = sub[4], *sub_rhoge = sub[5], *sub_rhogq_Lswp = sub[6], *sub_vx = sub[7];
  double *sub_vy = sub[8], *sub_vz = sub[9], *sub_w = sub[10], *sub_unccn = sub[11], *sub_rho = sub[12];
  double *sub_tem = sub[13], *sub_pre = sub[14], *sub_q_Lswp = sub[15], *sub_qd = sub[16];
  double *sub_precip_mp = sub[17], *sub_ISO1_precip = sub[18], *sub_ISO2_precip = sub[19];
  double *sub_rhoein_precip_mp = sub[20], *sub_lh_precip_mp = sub[21], *sub_rhophi_precip_mp = sub[22];
  double *sub_rhokin_precip_mp = sub[23], *sub_rceff = sub[24], *sub_rceff_solid = sub[25];
  double *sub_rceff_cld = sub[26], *sub_rctop = sub[27], *sub_rwtop = sub[28], *sub_tctop = sub[29];
  double *sub_frhoge_af = sub[30], *sub_frhogqv_af = sub[31], *sub_frhoge_rad = sub[32], *sub_qke = sub[33];
  double *sub_gsgam2 = sub[34], *sub_gsgam2h = sub[35], *sub_gam2 = sub[36], *sub_gam2h = sub[37];
  double *sub_ix = sub[38], *sub_iy = sub[39], *sub_iz = sub[40], *sub_jx = sub[41], *sub_jy = sub[42];
  double *sub_jz = sub[43], *sub_z = sub[44], *sub_zh = sub[45], *sub_GDCLW = sub[46], *sub_GDCFRC = sub[47];
  double *sub_GPREC = sub[48], *sub_CBMFX = sub[49];
  const double TIME_DTL = dt, TIME_CTIME = 0.0;

  nsw6_handle* h = nullptr;
  int rc = nsw6_create(&h, gall, kall, /*lall_max=*/1, gz.data(), gzh.data());
  if (rc != NSW6_OK) {
    std::fprintf(stderr, "nsw6_create: %s\n", nsw6_strerror(rc));
    return 4;
  }
  // precip rows of the [2][lall][1][gall] arrays are lall * gall apart
  rc = nsw6_set_precip_stride(h, (long long)lall * gall);
  if (rc == NSW6_OK)
    rc = mp_driver(h, l,
        sub_rhog, sub_rhogvx, sub_rhogvy, sub_rhogvz, sub_rhogw,
        sub_rhoge, sub_rhogq_Lswp, sub_vx, sub_vy, sub_vz, sub_w,
        sub_unccn, sub_rho, sub_tem, sub_pre, sub_q_Lswp, sub_qd,
        sub_precip_mp, sub_ISO1_precip, sub_ISO2_precip,
        sub_rhoein_precip_mp, sub_lh_precip_mp, sub_rhophi_precip_mp,
        sub_rhokin_precip_mp, sub_rceff, sub_rceff_solid, sub_rceff_cld,
        sub_rctop, sub_rwtop, sub_tctop, sub_frhoge_af, sub_frhogqv_af,
        sub_frhoge_rad, sub_qke, sub_gsgam2, sub_gsgam2h, sub_gam2,
        sub_gam2h, sub_ix, sub_iy, sub_iz, sub_jx, sub_jy,
        sub_jz, sub_z, sub_zh, TIME_DTL, TIME_CTIME,
        sub_GDCLW, sub_GDCFRC, sub_GPREC, sub_CBMFX);
  if (rc != NSW6_OK) {
    std::fprintf(stderr, "mp_driver: %s\n", nsw6_strerror(rc));
    return 5;
  }
  nsw6_destroy(h);

  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  for (int a = 0; a < 50; ++a) {
    const size_t n = host[a].size();
    if (!ok(cudaMemcpy(host[a].data(), dev[a], n * sizeof(double), cudaMemcpyDeviceToHost), "copy out")) return 3;
    std::fwrite(host[a].data(), sizeof(double), n, o);
    cudaFree(dev[a]);
  }
  std::fclose(o);
  std::printf("mp_driver region %d of %d: ok\n", l, lall);
  return 0;
}
