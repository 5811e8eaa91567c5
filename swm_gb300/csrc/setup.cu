// setup.cu -- host-side set-up of the device grid: the parts of the Fortran
// initialisation the accelerated path consumes, restated in C++ so that C and
// Python callers need no Fortran host (a Fortran host may pass the same
// values).  Time-stepping never runs here.
#include <cmath>
#include <cstring>
#include "ctx.h"

namespace swm {

// binary32-rounded PI: grid_module.f90:6-7 declares it with a default-real
// literal.
static const double kPI = (double)(float)3.14159265358979323846;

// initDomain: domain_module.f90:49-207; setLat/setf/setGridEuler:
// grid_module.f90:55-74, 116-145, 167-195.
int host_domain(swm_gpu_ctx *c, const double *Hin, const int8_t *Hmiss) {
  const swm_gpu_config &cf = c->cfg;
  HostGrid &g = c->hg;
  int nx = cf.nx, ny = cf.ny;
  size_t n = (size_t)nx * ny;
  g.nx = nx;
  g.ny = ny;
  g.D2R = kPI / 180.;
  g.dLambda = g.D2R * (cf.lon_e - cf.lon_s) / (nx - 1);
  g.dTheta = g.D2R * (cf.lat_e - cf.lat_s) / (ny - 1);
  auto ip1 = [nx](int i) { return i + 1 == nx ? 0 : i + 1; };
  auto jp1 = [ny](int j) { return j + 1 == ny ? 0 : j + 1; };
  for (int q = 0; q < 4; q++) {
    g.lat[q].assign(ny, 0.);
    g.lon[q].assign(nx, 0.);
    g.ocean[q].assign(n, 0);
    g.H[q].assign(n, 0.);
  }
  // coordinate vectors (:120-127); 2.*(N-1) is a default-real product
  const double hy = (cf.lat_e - cf.lat_s) / (double)(float)(2.f * (ny - 1));
  const double hx = (cf.lon_e - cf.lon_s) / (double)(float)(2.f * (nx - 1));
  for (int j = 0; j < ny; j++) {
    double lv = j * (cf.lat_e - cf.lat_s) / (ny - 1) + cf.lat_s;
    g.lat[GV][j] = lv;
    g.lat[GH][j] = lv;
    g.lat[GU][j] = lv + hy;
    g.lat[GE][j] = lv + hy;
  }
  for (int i = 0; i < nx; i++) {
    double lh = i * (cf.lon_e - cf.lon_s) / (nx - 1) + cf.lon_s;
    g.lon[GH][i] = lh;
    g.lon[GU][i] = lh;
    g.lon[GV][i] = lh + hx;
    g.lon[GE][i] = lh + hx;
  }
  // bathymetry (:130-151)
  std::vector<double> &H = g.H[GH];
  if (Hin) {
    for (size_t k = 0; k < n; k++) {
      H[k] = Hin[k];
      if (Hmiss && Hmiss[k]) H[k] = 0.;
      if (H[k] <= 0.) H[k] = 0.;
    }
  } else {
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) H[i + (size_t)nx * j] = (i == 0 || i == nx - 1) ? 0. : 1.;
  }
  for (int i = 0; i < nx; i++) {
    H[i] = 0.;
    H[i + (size_t)nx * (ny - 1)] = 0.;
  }
  // masks (:156-172)
  std::vector<int8_t> &oH = g.ocean[GH], &oU = g.ocean[GU], &oV = g.ocean[GV], &oE = g.ocean[GE];
  for (size_t k = 0; k < n; k++) oH[k] = (H[k] == 0.) ? 0 : 1;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      size_t k = i + (size_t)nx * j;
      int lH = 1 - oH[k], lHj = 1 - oH[i + (size_t)nx * jp1(j)];
      int lHi = 1 - oH[ip1(i) + (size_t)nx * j], lHij = 1 - oH[ip1(i) + (size_t)nx * jp1(j)];
      oU[k] = (lH + lHj == 2) ? 0 : 1;
      oV[k] = (lH + lHi == 2) ? 0 : 1;
      oE[k] = (lH + lHj + lHi + lHij == 4) ? 0 : 1;
    }
  // depth on all grids (:177-193)
  std::vector<double> &Hu = g.H[GU], &Hv = g.H[GV], &He = g.H[GE];
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      size_t k = i + (size_t)nx * j, ki = ip1(i) + (size_t)nx * j, kj = i + (size_t)nx * jp1(j);
      size_t kij = ip1(i) + (size_t)nx * jp1(j);
      if (oU[k]) Hu[k] = (H[k] + H[kj]) / (double)(oH[k] + oH[kj]);
      if (oV[k]) Hv[k] = (H[k] + H[ki]) / (double)(oH[k] + oH[ki]);
      if (oE[k]) He[k] = (H[k] + H[ki] + H[kj] + H[kij]) / (double)(oH[k] + oH[ki] + oH[kj] + oH[kij]);
    }
  if (cf.H_overwrite != 0.) {
    for (size_t k = 0; k < n; k++) {
      H[k] = oH[k] * cf.H_overwrite;
      Hu[k] = oU[k] * cf.H_overwrite;
      Hv[k] = oV[k] * cf.H_overwrite;
      He[k] = oE[k] * cf.H_overwrite;
    }
  }
  // metric and Coriolis parameter per grid
  double rtheta0 = cf.theta0 * g.D2R;
  for (int q = 0; q < 4; q++) {
    g.sinl[q].resize(ny);
    g.cosl[q].resize(ny);
    g.tanl[q].resize(ny);
    g.f[q].resize(ny);
    for (int j = 0; j < ny; j++) {
      double r = g.lat[q][j] * g.D2R;
      g.sinl[q][j] = std::sin(r);
      g.cosl[q][j] = std::cos(r);
      g.tanl[q][j] = std::tan(r);
      double fv = 0.;
      switch (cf.coriolis_approx) {
        case 1: fv = 2 * cf.OMEGA * std::sin(rtheta0); break;
        case 2: fv = 2 * cf.OMEGA * std::sin(rtheta0) + 2 * cf.OMEGA * std::cos(rtheta0) * (g.D2R * g.lat[q][j]); break;
        case 3: fv = 2 * cf.OMEGA * g.sinl[q][j]; break;
        default: fv = 0.; break;
      }
      g.f[q][j] = fv;
    }
  }
  for (int q = 0; q < 3; q++) {
    g.glin[q].assign(n, 0.);
    g.impl[q].assign(n, 1.);
  }
  for (int q = 0; q < 2; q++) g.gsq[q].assign(n, 0.);
  return SWM_GPU_OK;
}

// evaluateStreamfunction2D (calc_lib.f90:812-878) and laplacian2D
// (calc_lib.f90:1174-1206) of the basic-state streamfunction, as
// SWM_timestep_init does for LINEARISED_MEAN_STATE (:73-85).
void host_basic_state(swm_gpu_ctx *c, const double *psi_in) {
  HostGrid &g = c->hg;
  const swm_gpu_config &cf = c->cfg;
  int nx = g.nx, ny = g.ny;
  size_t n = (size_t)nx * ny;
  std::vector<double> psi(psi_in, psi_in + n);
  if (cf.mask_psi_bs)
    for (size_t k = 0; k < n; k++) psi[k] = psi[k] * g.ocean[GH][k];
  g.ubs.assign(n, 0.);
  g.vbs.assign(n, 0.);
  g.zbs.assign(n, 0.);
  const std::vector<int8_t> &oH = g.ocean[GH], &oU = g.ocean[GU], &oV = g.ocean[GV];
  auto bc = [&](int q, size_t k) { return g.ocean[q][k] == 1 ? 1. : cf.lbc; };
  double A = cf.A, dL = g.dLambda, dT = g.dTheta;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      int ip = i + 1 == nx ? 0 : i + 1, jp = j + 1 == ny ? 0 : j + 1;
      size_t k = i + (size_t)nx * j, kj = i + (size_t)nx * jp, ki = ip + (size_t)nx * j;
      double dy = (oH[kj] + oH[k] == 0) ? 0. : bc(GU, k) * (psi[kj] - psi[k]) / (A * dT);
      g.ubs[k] = -dy;
      if (cf.barotropic && oU[k] == 1) g.ubs[k] = g.ubs[k] / g.H[GU][k];
      double dx = (oH[ki] + oH[k] == 0) ? 0. : bc(GV, k) / (A * g.cosl[GV][j] * dL) * (psi[ki] - psi[k]);
      g.vbs[k] = dx;
      if (cf.barotropic && oV[k] == 1) g.vbs[k] = g.vbs[k] / g.H[GV][k];
    }
  const std::vector<double> &cH = g.cosl[GH];
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      size_t k = i + (size_t)nx * j;
      if (oH[k] != 1) continue;
      int ip = i + 1 == nx ? 0 : i + 1, im = i == 0 ? nx - 1 : i - 1;
      int jp = j + 1 == ny ? 0 : j + 1, jm = j == 0 ? ny - 1 : j - 1;
      size_t kip = ip + (size_t)nx * j, kim = im + (size_t)nx * j;
      size_t kjp = i + (size_t)nx * jp, kjm = i + (size_t)nx * jm;
      double t1 = 1 / ((A * cH[j] * dL) * (A * cH[j] * dL)) *
                  (bc(GV, k) * (psi[kip] - psi[k]) - bc(GV, kim) * (psi[k] - psi[kim]));
      double t2 = 1 / (A * A * cH[j] * (dT * dT)) *
                  (bc(GU, k) * (cH[jp] * psi[kjp] - cH[j] * psi[k]) -
                   bc(GU, kjm) * (cH[j] * psi[k] - cH[jm] * psi[kjm]));
      g.zbs[k] = t1 + t2;
    }
}

// getDampingCoefficient (swm_damping_module.f90:137-203) and getSpongeLayer
// (:257-359, SPONGE_SCALE_UNIT = SCU_DEGREE).  damping_additive reproduces the
// older selfcheck build in which namelist records add up.
void host_damping_add(swm_gpu_ctx *c, int term, int type, double value, double sl_length,
                      double sl_cutoff, int loc, const double *file_data) {
  HostGrid &g = c->hg;
  int nx = g.nx, ny = g.ny;
  size_t n = (size_t)nx * ny;
  std::vector<double> *target;
  int grid;
  switch (term) {
    case SWM_TERM_GAMMA_LIN_U: target = &g.glin[0]; grid = GU; break;
    case SWM_TERM_GAMMA_LIN_V: target = &g.glin[1]; grid = GV; break;
    case SWM_TERM_GAMMA_LIN_ETA: target = &g.glin[2]; grid = GE; break;
    case SWM_TERM_GAMMA_SQ_U: target = &g.gsq[0]; grid = GU; break;
    default: target = &g.gsq[1]; grid = GV; break;
  }
  std::vector<double> fresh;
  std::vector<double> *coef = target;
  if (c->cfg.damping_additive) {
    fresh.assign(n, 0.);
    coef = &fresh;
  }
  std::vector<double> &C = *coef;
  if (type == SWM_DAMP_UNIFORM) {
    for (size_t k = 0; k < n; k++) C[k] = std::fmax(C[k], value);
  } else if (type == SWM_DAMP_FILE) {
    for (size_t k = 0; k < n; k++) C[k] = std::fmax(file_data[k], C[k]);
  } else {
    const double D2R = kPI / 180.;
    double sc = D2R * c->cfg.A / sl_length / (D2R * c->cfg.A);
    // iSponge(boundary, grid), 1-based: S, N, W, E
    int iS[3][4] = {{1, ny - 1, 2, nx - 1}, {2, ny - 1, 1, nx - 1}, {1, ny - 1, 1, nx - 1}};
    int *is = iS[grid - 1];
    const std::vector<double> &lat = g.lat[grid], &lon = g.lon[grid];
    double ecut = std::exp(-sl_cutoff);
    auto row = [&](double lb) {
      for (int j = 0; j < ny; j++) {
        double v = value * (std::exp(-std::fabs(lat[j] - lb) * sc) - ecut);
        for (int i = 0; i < nx; i++) C[i + (size_t)nx * j] = std::fmax(v, C[i + (size_t)nx * j]);
      }
    };
    auto col = [&](double lb) {
      for (int i = 0; i < nx; i++) {
        double v = value * (std::exp(-std::fabs(lon[i] - lb) * sc) - ecut);
        for (int j = 0; j < ny; j++) C[i + (size_t)nx * j] = std::fmax(v, C[i + (size_t)nx * j]);
      }
    };
    if (loc & SWM_SPONGE_N) row(lat[is[1] - 1]);
    if (loc & SWM_SPONGE_S) row(lat[is[0] - 1]);
    if (loc & SWM_SPONGE_W) col(lon[is[2] - 1]);
    if (loc & SWM_SPONGE_E) col(lon[is[3] - 1]);
  }
  if (coef != target)
    for (size_t k = 0; k < n; k++) (*target)[k] = (*target)[k] + C[k];
}

// tail of SWM_damping_init (swm_damping_module.f90:78-115).  g.H holds the
// depths after computeD at itt=0 (the device overwrote H_u/H_v in linear
// modes; the caller refreshed g.H from the device).
void host_damping_finish(swm_gpu_ctx *c) {
  HostGrid &g = c->hg;
  size_t n = (size_t)g.nx * g.ny;
  const swm_gpu_config &cf = c->cfg;
  if (cf.barotropic) {
    for (size_t k = 0; k < n; k++) {
      if (g.ocean[GU][k] == 1) g.glin[0][k] = g.glin[0][k] / g.H[GU][k];
      if (g.ocean[GV][k] == 1) g.glin[1][k] = g.glin[1][k] / g.H[GV][k];
    }
    if (cf.quadratic_friction)
      for (size_t k = 0; k < n; k++) {
        if (g.ocean[GU][k] == 1) g.gsq[0][k] = g.gsq[0][k] / g.H[GU][k];
        if (g.ocean[GV][k] == 1) g.gsq[1][k] = g.gsq[1][k] / g.H[GV][k];
      }
  }
  for (size_t k = 0; k < n; k++) {
    g.impl[0][k] = 1. + cf.dt * g.glin[0][k];
    g.impl[1][k] = 1. + cf.dt * g.glin[1][k];
    g.impl[2][k] = 1. + cf.dt * g.glin[2][k];
  }
}

// computeStreamfunction (calc_lib.f90:727-780) without an elliptic solver
// configured (u_nd = u).  Row/column prefix sums in the reference's order.

}  // namespace swm
