// plain.cu -- FP64 per-module kernels: the drop-in path.
//
// One kernel per reference loop nest, same formulas, same evaluation order;
// this translation unit is compiled with -fmad=false so that every product
// and sum is rounded exactly as the FP64 CPU restatement rounds it.  Fields
// are unpadded (Nx, Ny); neighbour indices wrap periodically like the
// reference's cshift index vectors (domain_module.f90:106-115).
#include "ctx.h"
#include "divide.cuh"

namespace swm {

#define IDX(i, j) ((size_t)(i) + (size_t)d.nx * (size_t)(j))

__device__ __forceinline__ int ip1(int i, int n) { return i + 1 == n ? 0 : i + 1; }
__device__ __forceinline__ int im1(int i, int n) { return i == 0 ? n - 1 : i - 1; }

// 1 / max(count, 1) for a count of ocean points 0..4: the reference's
// division, taken from its correctly rounded values (1/3 is the constant the
// division by 3 rounds to)
__device__ __forceinline__ double inv_count(int n) { return n >= 4 ? .25 : (n == 3 ? 1. / 3. : (n == 2 ? .5 : 1.)); }

// mask-normalised interpolation weights (calc_lib.f90:253-265, 320-335):
// the mask (0 or 1) times the weight is the weight or +0, as the product
// rounds, taken by a select
__device__ __forceinline__ double mw(int8_t m, double w) { return m ? w : 0.; }
__device__ __forceinline__ double ip2_noland(const double *v, const int8_t *m, size_t k1, size_t k2) {
  double w = inv_count(m[k1] + m[k2]);
  return mw(m[k1], w) * v[k1] + mw(m[k2], w) * v[k2];
}
__device__ __forceinline__ double ip4_noland(const double *v, const int8_t *m, size_t k1, size_t k2,
                                             size_t k3, size_t k4) {
  double w = inv_count(m[k1] + m[k2] + m[k3] + m[k4]);
  return mw(m[k1], w) * v[k1] + mw(m[k2], w) * v[k2] + mw(m[k3], w) * v[k3] + mw(m[k4], w) * v[k4];
}
__device__ __forceinline__ double ip2(const double *v, size_t k1, size_t k2) { return .5 * v[k1] + .5 * v[k2]; }
__device__ __forceinline__ double ip4(const double *v, size_t k1, size_t k2, size_t k3, size_t k4) {
  return .25 * v[k1] + .25 * v[k2] + .25 * v[k3] + .25 * v[k4];
}

#define KERNEL_PROLOGUE                               \
  int i = blockIdx.x * blockDim.x + threadIdx.x;      \
  int j = blockIdx.y * blockDim.y + threadIdx.y;      \
  if (i >= d.nx || j >= d.ny) return;                \
  size_t k = IDX(i, j);

// computeD, FULLY_NONLINEAR part (swm_nonlinear_timestep_module.f90:187-197)
__global__ void k_D_nonlinear(Dev d) {
  KERNEL_PROLOGUE
  if (d.ocean[GE][k] != 1) return;
  d.D[k] = d.eta0[k] + d.Hg[GE][k];
}

// computeD, thickness on H/u/v points (:201-217)
__global__ void k_D_interp(Dev d) {
  KERNEL_PROLOGUE
  const int8_t *oE = d.ocean[GE];
  int im = im1(i, d.nx), jm = im1(j, d.ny);
  double dh = ip4_noland(d.D, oE, k, IDX(im, jm), IDX(im, j), IDX(i, jm));
  double du = ip2_noland(d.D, oE, k, IDX(im, j));
  double dv = ip2_noland(d.D, oE, k, IDX(i, jm));
  d.Dh[k] = dh;
  d.Du[k] = du;
  d.Dv[k] = dv;
}

// The plain path's fixed divisors per row (plain_prepare): PROW_N doubles,
// the divisor and its reciprocal for A cos_eta (continuity), A cos_u dLambda
// (zonal pressure gradient) and cos_H (vorticity), then the vorticity's
// factors bc / (A cos_H dLambda) for bc = 1 and bc = lbc.  Divisions by them
// go through div_fast (divide.cuh): the quotients are the division
// operator's, bit for bit.
constexpr int PROW_N = 8;

__global__ void k_plain_rows(Dev d, double *prow, int *bad) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.ny) return;
  double *P = prow + (size_t)PROW_N * j;
  const double bE = d.A * d.cosl[GE][j], bU = d.A * d.cosl[GU][j] * d.dLambda, cH = d.cosl[GH][j];
  P[0] = bE; P[1] = 1. / bE;
  P[2] = bU; P[3] = 1. / bU;
  P[4] = cH; P[5] = 1. / cH;
  P[6] = 1. / (d.A * d.cosl[GH][j] * d.dLambda);
  P[7] = d.lbc / (d.A * d.cosl[GH][j] * d.dLambda);
  if (!div_rn_range(bE) || !div_rn_range(bU) || !div_rn_range(cH)) atomicOr(bad, 1);
}

// 1 / impl per point; every point's impl in div_fast's range
__global__ void k_plain_rimpl(Dev d, double *r0, double *r1, double *r2, int *bad) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)d.nx * d.ny) return;
  const double a = d.impl_u[k], b = d.impl_v[k], e = d.impl_e[k];
  r0[k] = 1. / a;
  r1[k] = 1. / b;
  r2[k] = 1. / e;
  if (!div_rn_range(a) || !div_rn_range(b) || !div_rn_range(e)) atomicOr(bad, 1);
}

// computeRelVort -> vorticityFromVelocities2D (calc_lib.f90:663-678)
__global__ void k_vorticity(Dev d) {
  KERNEL_PROLOGUE
  size_t ki = IDX(im1(i, d.nx), j), kj = IDX(i, im1(j, d.ny));
  const bool ocean_h = d.ocean[GH][k] == 1;
  double bc = ocean_h ? 1. : d.lbc;
  const double *P = d.prow + (size_t)PROW_N * j;
  double dvdx, dudy;
  if (d.ocean[GV][ki] + d.ocean[GV][k] == 0) dvdx = 0.;
  else dvdx = (d.pdiv ? P[ocean_h ? 6 : 7] : bc / (d.A * d.cosl[GH][j] * d.dLambda)) * (d.v0[k] - d.v0[ki]);
  if (d.ocean[GU][k] + d.ocean[GU][kj] == 0) {
    dudy = 0.;
  } else {
    const double num = bc * (d.cosl[GU][j] * d.u0[k] - d.cosl[GU][im1(j, d.ny)] * d.u0[kj]);
    dudy = d.pdiv ? div_fast(num, d.AdT, d.r_AdT) : num / (d.A * d.dTheta);
  }
  d.zeta[k] = dvdx - (d.pdiv ? div_fast(dudy, P[4], P[5]) : dudy / d.cosl[GH][j]);
}

// computePotVort (:230-257)
__global__ void k_pot(Dev d) {
  KERNEL_PROLOGUE
  const double eps = 2.220446049250313e-16;
  double pD = fmax(d.Dh[k], eps);
  double fH = d.f[GH][j];
  if (d.mode == SWM_MODE_NONLINEAR) d.pot[k] = (fH + d.zeta[k]) / pD;
  else if (d.mode == SWM_MODE_LIN_MEAN) d.pot[k] = (fH + d.zbs[k]) / pD;
  else d.pot[k] = fH / pD;
}

// computeEdens (:259-310); u2/v2 of the reference evaluated in place
__global__ void k_edens(Dev d) {
  KERNEL_PROLOGUE
  if (d.ocean[GE][k] != 1) return;
  size_t ku = IDX(ip1(i, d.nx), j), kv = IDX(i, ip1(j, d.ny));
  if (d.mode == SWM_MODE_NONLINEAR) {
    double a = .5 * (d.u0[ku] * d.u0[ku]) + .5 * (d.u0[k] * d.u0[k]);
    double b = .5 * (d.v0[kv] * d.v0[kv]) + .5 * (d.v0[k] * d.v0[k]);
    d.edens[k] = (a + b) * .5 + d.G * d.eta0[k];  // halving: the same rounding as / 2
  } else if (d.mode == SWM_MODE_LIN_MEAN) {
    double a = .5 * (d.u0[ku] * d.ubs[ku]) + .5 * (d.u0[k] * d.ubs[k]);
    double b = .5 * (d.v0[kv] * d.vbs[kv]) + .5 * (d.v0[k] * d.vbs[k]);
    d.edens[k] = (a + b) + d.G * d.eta0[k];
  } else {
    d.edens[k] = d.G * d.eta0[k];
  }
}

// computeMassFluxes (:312-326)
__global__ void k_massflux(Dev d) {
  KERNEL_PROLOGUE
  if (d.ocean[GU][k] == 1) d.mu[k] = d.Du[k] * d.u0[k];
  if (d.ocean[GV][k] == 1) d.mv[k] = d.Dv[k] * d.v0[k];
}

// Lateral-mixing coefficients of _init_p_coefficients (:132-145) and
// lat_mixing_u/v (:84-97).  They depend on the row (cos and tan of the
// latitude) and on two mask bits of the point, so they are formed once per
// row and mask case by the same expressions, in the same order, and the
// step kernels look them up: the values are bit for bit those formed per
// point (this file is compiled without FMA contraction).
constexpr int LATP_N = 14;  // pll: c0, c1[3], c2[3]; plt: c0, c1[3], c2[3]
constexpr int LATUV_N = 10; // lu: c0, c1[2], c2[2]; lv: c0, c1[2], c2[2]

// case of a coefficient that carries mask bit a (with neighbour bit b) in
// the term a * tan / max(a + b, 1): 0 when a = 0, 1 + b otherwise
__device__ __forceinline__ int latp_case(int a, int b) { return a ? 1 + b : 0; }

__global__ void k_latmix_tab_p(Dev d, double Ah, double *tab) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.ny) return;
  const double A = d.A, bc = 1.;
  double *T = tab + (size_t)LATP_N * j;
  for (int q = 0; q < 3; q++) {  // mask cases (own bit, other bit): (0, 0), (1, 0), (1, 1)
    const int8_t a = q > 0, b = q > 1;
    {  // pll: c1 carries ovp (a), c2 carries ov (a)
      const int o = a + b;
      const double ot = (double)(o > 1 ? o : 1), tn = d.tanl[GE][j];
      T[1 + q] = Ah / A * (bc / d.dTheta + a * tn / ot);
      T[4 + q] = Ah / A * (-bc / d.dTheta + a * tn / ot);
    }
    {  // plt: c1 carries ou (a), c2 carries oum (a)
      const int o = a + b;
      const double ot = (double)(o > 1 ? o : 1), tn = d.tanl[GH][j];
      T[8 + q] = -Ah / A * (bc / d.dTheta + a * tn / ot);
      T[11 + q] = -Ah / A * (-bc / d.dTheta + a * tn / ot);
    }
  }
  T[0] = -Ah * bc / d.dLambda / A / d.cosl[GE][j];
  T[7] = -Ah * bc / d.dLambda / A / d.cosl[GH][j];
}

__global__ void k_latmix_tab_uv(Dev d, double *tab) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.ny) return;
  const double A = d.A, bc = 1.;
  double *T = tab + (size_t)LATUV_N * j;
  for (int q = 0; q < 2; q++) {  // ot = 1, 2
    const double ot = (double)(q + 1);
    const double tu = d.tanl[GU][j], tv = d.tanl[GV][j];
    T[1 + q] = -(bc / A / d.dTheta - 2. * tu / A / ot);
    T[3 + q] = -(-bc / A / d.dTheta - 2. * tu / A / ot);
    T[6 + q] = -(-bc / A / d.dTheta + 2. * tv / A / ot);
    T[8 + q] = -(bc / A / d.dTheta + 2. * tv / A / ot);
  }
  T[0] = -bc / A / d.cosl[GU][j] / d.dLambda;
  T[5] = -bc / A / d.cosl[GV][j] / d.dLambda;
}

// SWM_LateralMixing_compute_p (swm_lateralmixing_module.f90:215-240), the
// coefficients from the table of this Ah
__global__ void k_latmix_p(Dev d, const double *__restrict__ tab, const double *u, const double *v,
                           const double *Dp, const double *Dhp, double *pll, double *plt) {
  KERNEL_PROLOGUE
  const double *T = tab + (size_t)LATP_N * j;
  if (d.ocean[GE][k] == 1) {
    size_t kjp = IDX(i, ip1(j, d.ny));
    int8_t ov = d.ocean[GV][k], ovp = d.ocean[GV][kjp];
    double c0 = T[0], c1 = T[1 + latp_case(ovp, ov)], c2 = T[4 + latp_case(ov, ovp)];
    pll[k] = Dp[k] * (c0 * (u[IDX(ip1(i, d.nx), j)] - u[k]) + c1 * v[kjp] + c2 * v[k]);
  }
  if (d.ocean[GH][k] == 1) {
    size_t kjm = IDX(i, im1(j, d.ny));
    int8_t ou = d.ocean[GU][k], oum = d.ocean[GU][kjm];
    double c0 = T[7], c1 = T[8 + latp_case(ou, oum)], c2 = T[11 + latp_case(oum, ou)];
    plt[k] = Dhp[k] * (c0 * (v[k] - v[IDX(im1(i, d.nx), j)]) + c1 * u[k] + c2 * u[kjm]);
  }
}

// SWM_LateralMixing_compute_uv (:162-186) with lat_mixing_u/v (:84-97) from
// the table
// unit: the thicknesses are 1 (the biharmonic operator's first pass), and
// x / 1 = x exactly
__global__ void k_latmix_uv(Dev d, const double *__restrict__ tab, const double *pll, const double *plt,
                            const double *Dup, const double *Dvp, double *lu, double *lv, int unit) {
  KERNEL_PROLOGUE
  const double *T = tab + (size_t)LATUV_N * j;
  if (d.ocean[GU][k] == 1) {
    const int q = d.ocean[GH][k] + d.ocean[GH][IDX(i, ip1(j, d.ny))] > 1;
    double c0 = T[0], c1 = T[1 + q], c2 = T[3 + q];
    const double x = c0 * (pll[k] - pll[IDX(im1(i, d.nx), j)]) + c1 * plt[IDX(i, ip1(j, d.ny))] + c2 * plt[k];
    lu[k] = unit ? x : x / Dup[k];
  }
  if (d.ocean[GV][k] == 1) {
    const int q = d.ocean[GE][k] + d.ocean[GE][IDX(i, im1(j, d.ny))] > 1;
    double c0 = T[5], c1 = T[6 + q], c2 = T[8 + q];
    const double x = c0 * (plt[IDX(ip1(i, d.nx), j)] - plt[k]) + c1 * pll[k] + c2 * pll[IDX(i, im1(j, d.ny))];
    lv[k] = unit ? x : x / Dvp[k];
  }
}

// SWM_timestep_nonlinear, continuity (:349-374)
__global__ void k_tend_eta(Dev d) {
  KERNEL_PROLOGUE
  if (d.ocean[GE][k] != 1) return;
  int ip = ip1(i, d.nx), jp = ip1(j, d.ny);
  const double *cV = d.cosl[GV];
  auto dL = [&](double x) { return d.pdiv ? div_fast(x, d.dLambda, d.r_dLambda) : x / d.dLambda; };
  auto dT = [&](double x) { return d.pdiv ? div_fast(x, d.dTheta, d.r_dTheta) : x / d.dTheta; };
  double t = dL(-(d.mu[IDX(ip, j)] - d.mu[k])) - dT(d.mv[IDX(i, jp)] * cV[jp] - d.mv[k] * cV[j]);
  if (d.mode == SWM_MODE_LIN_MEAN) {
    const int8_t *oE = d.ocean[GE];
    int qi = ip1(j % d.nx, d.nx);  // ip1(j): zonal index taken from j in the reference (:360)
    double ea = ip2_noland(d.eta0, oE, IDX(qi, j), IDX(im1(qi, d.nx), j));
    double eb = ip2_noland(d.eta0, oE, k, IDX(im1(i, d.nx), j));
    double ec = ip2_noland(d.eta0, oE, IDX(i, jp), IDX(i, im1(jp, d.ny)));
    double ed = ip2_noland(d.eta0, oE, k, IDX(i, im1(j, d.ny)));
    t = t - dL(ea * d.ubs[IDX(ip, j)] - eb * d.ubs[k]) - dT(cV[jp] * ec * d.vbs[IDX(i, jp)] - cV[j] * ed * d.vbs[k]);
  }
  const double *P = d.prow + (size_t)PROW_N * j;
  d.Ge[2][k] = (d.pdiv ? div_fast(t, P[0], P[1]) : t / (d.A * d.cosl[GE][j])) + d.Fe[k];
}

// SWM_timestep_nonlinear, zonal momentum (:378-409)
__global__ void k_tend_u(Dev d) {
  KERNEL_PROLOGUE
  if (d.ocean[GU][k] != 1) return;
  int im = im1(i, d.nx), jp = ip1(j, d.ny);
  size_t a1 = IDX(i, jp), a2 = IDX(im, j), a3 = IDX(im, jp);
  double g = ip2(d.pot, a1, k) * ip4(d.mv, a1, a2, a3, k);
  if (d.mode == SWM_MODE_LIN_MEAN) g = g + ip2(d.zeta, a1, k) * ip4(d.vbs, a1, a2, a3, k);
  const double *P = d.prow + (size_t)PROW_N * j;
  const double de = d.edens[k] - d.edens[IDX(im, j)];
  g = g - (d.pdiv ? div_fast(de, P[2], P[3]) : de / (d.A * d.cosl[GU][j] * d.dLambda));
  if (d.qbf) {
    double vv = ip4(d.v0, a1, a2, a3, k);
    double q = d.gsq_u[k] * sqrt(d.u0[k] * d.u0[k] + (vv * vv)) * d.u0[k];
    if (d.barotropic) q = q / d.Hg[GU][k];
    g = g - q;
  }
  if (d.lateral_mixing) g = g + d.lmu[k];
  d.Gu[2][k] = g + d.Fx[k];
}

// SWM_timestep_nonlinear, meridional momentum (:411-444)
__global__ void k_tend_v(Dev d) {
  KERNEL_PROLOGUE
  if (d.ocean[GV][k] != 1) return;
  int ip = ip1(i, d.nx), jm = im1(j, d.ny);
  size_t a1 = IDX(ip, j), a2 = IDX(i, jm), a4 = IDX(ip, jm);
  double g = -ip2(d.pot, a1, k) * ip4(d.mu, a1, a2, k, a4);
  if (d.mode == SWM_MODE_LIN_MEAN) g = g - ip2(d.zeta, a1, k) * ip4(d.ubs, a1, a2, k, a4);
  const double de = d.edens[k] - d.edens[IDX(i, jm)];
  g = g - (d.pdiv ? div_fast(de, d.AdT, d.r_AdT) : de / (d.A * d.dTheta));
  if (d.qbf) {
    double uu = ip4(d.u0, a1, a2, k, a4);
    double q = d.gsq_v[k] * sqrt(d.v0[k] * d.v0[k] + (uu * uu)) * d.v0[k];
    if (d.barotropic) q = q / d.Hg[GV][k];
    g = g - q;
  }
  if (d.lateral_mixing) g = g + d.lmv[k];
  d.Gv[2][k] = g + d.Fy[k];
}

struct ABCoef {
  double c[3];
  double dtc[3];  // dt * c[t], the product the reference forms first (host, the same rounding)
  int tstep;
};

// integrate_AB_vec (time_integration_module.f90:74-112) for the three
// prognostic fields, plus the FULLY_NONLINEAR thickness clamp (:176-179)
__global__ void k_integrate(Dev d, ABCoef ab) {
  KERNEL_PROLOGUE
  double a = d.eta0[k], b = d.u0[k], c = d.v0[k];
  for (int t = 0; t < ab.tstep; t++) {
    a = a + ab.dtc[t] * d.Ge[t][k];
    b = b + ab.dtc[t] * d.Gu[t][k];
    c = c + ab.dtc[t] * d.Gv[t][k];
  }
  a = d.pdiv ? div_fast(a, d.impl_e[k], d.rimpl[2][k]) : a / d.impl_e[k];
  if (d.mode == SWM_MODE_NONLINEAR) {
    double lim = d.minD - d.Hg[GE][k];
    if (a < lim) a = lim;
  }
  d.eta1[k] = a;
  d.u1[k] = d.pdiv ? div_fast(b, d.impl_u[k], d.rimpl[0][k]) : b / d.impl_u[k];
  d.v1[k] = d.pdiv ? div_fast(c, d.impl_v[k], d.rimpl[1][k]) : c / d.impl_v[k];
}

// SWM_forcing_update reset (swm_forcing_module.f90:141-149)
__global__ void k_forcing_reset(Dev d) {
  KERNEL_PROLOGUE
  d.Fe[k] = d.Fec[k];
  d.Fx[k] = d.Fxc[k];
  d.Fy[k] = d.Fyc[k];
}

// SWM_forcing_process* for one stream (swm_forcing_module.f90:274-552)
__global__ void k_stream(Dev d, Stream s, double *Fx, double *Fy, double *Fe, double r_iot, double i_iot) {
  KERNEL_PROLOGUE
  const int8_t *oU = d.ocean[GU], *oV = d.ocean[GV], *oE = d.ocean[GE];
  const double *dd = s.d1;
  switch (s.type) {
    case SWM_FRC_WIND: {
      bool z = s.comp == SWM_CMP_ZONAL;
      double *F = z ? Fx : Fy;
      const int8_t *m = z ? oU : oV;
      const double *H = z ? d.Du : d.Dv;
      bool sh = d.barotropic || d.mode == SWM_MODE_NONLINEAR;
      if (m[k] == 1) F[k] = F[k] + (d.tau_scale * dd[k] / (sh ? (d.RHO0 * H[k]) : d.RHO0));
      break;
    }
    case SWM_FRC_OSC: {
      double *F = s.comp == SWM_CMP_ZONAL ? d.Fx : (s.comp == SWM_CMP_MERID ? d.Fy : d.Fe);
      const int8_t *m = s.comp == SWM_CMP_ZONAL ? oU : (s.comp == SWM_CMP_MERID ? oV : oE);
      F[k] = F[k] + (2. * (s.d1[k] * r_iot - s.d2[k] * i_iot)) * m[k];
      break;
    }
    case SWM_FRC_CUSTOM: {
      double *F = s.comp == SWM_CMP_ZONAL ? Fx : (s.comp == SWM_CMP_MERID ? Fy : Fe);
      const int8_t *m = s.comp == SWM_CMP_ZONAL ? oU : (s.comp == SWM_CMP_MERID ? oV : oE);
      if (m[k] == 1) F[k] = F[k] + dd[k];
      break;
    }
    case SWM_FRC_HEAT:
      if (oE[k] == 1) Fe[k] = Fe[k] + dd[k];
      break;
    case SWM_FRC_EMF: {
      double A = d.A;
      const double *He = d.Hg[GE], *Hu = d.Hg[GU], *Hv = d.Hg[GV], *H = d.Hg[GH];
      const double *cu = d.cosl[GU], *cv = d.cosl[GV];
      int nx = d.nx, ny = d.ny;
      auto h2eta = [&](int ii, int jj) {
        return ip4(dd, IDX(ip1(ii, nx), ip1(jj, ny)), IDX(ii, jj), IDX(ii, ip1(jj, ny)), IDX(ip1(ii, nx), jj));
      };
      if (s.comp == SWM_CMP_U2) {
        if (oU[k] != 1) break;
        int im = im1(i, nx);
        Fx[k] = Fx[k] + (-(h2eta(i, j) * He[k] - h2eta(im, j) * He[IDX(im, j)]) / (2 * A * d.dLambda * cu[j] * Hu[k]));
      } else if (s.comp == SWM_CMP_V2) {
        if (oV[k] != 1) break;
        int jm = im1(j, ny);
        Fy[k] = Fy[k] + (-(cu[j] * He[k] * h2eta(i, j) - cu[jm] * He[IDX(i, jm)] * h2eta(i, jm)) /
                         (8 * A * d.dTheta * cv[j] * Hv[k]));
      } else {
        int jp = ip1(j, ny), ip = ip1(i, nx);
        if (oU[k] == 1)
          Fx[k] = Fx[k] + (-(cv[jp] * dd[IDX(i, jp)] * H[IDX(i, jp)] - cv[j] * dd[k] * H[k]) /
                           (2 * A * d.dTheta * cu[j] * Hu[k]));
        if (oV[k] == 1)
          Fy[k] = Fy[k] + (-(dd[IDX(ip, j)] * H[IDX(ip, j)] - dd[k] * H[k]) / (2 * A * d.dLambda * cv[j] * Hv[k]));
      }
      break;
    }
  }
}

__global__ void k_fill(double *p, size_t n, double v) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) p[k] = v;
}

#undef KERNEL_PROLOGUE

static dim3 blk() { return dim3(32, 8); }
static dim3 grd(const swm_gpu_ctx *c) { return dim3((c->nx + 31) / 32, (c->ny + 7) / 8); }

#define LAUNCH(kern, ...)                                               \
  do {                                                                  \
    kern<<<grd(c), blk(), 0, c->stream>>>(__VA_ARGS__);                 \
    c->launches++;                                                      \
  } while (0)

int plain_fill(swm_gpu_ctx *c, double *p, double value) {
  k_fill<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(p, c->n, value);
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// SWM_timestep_advance diagnostics (swm_nonlinear_timestep_module.f90:150-154)
int plain_diagnostics(swm_gpu_ctx *c, int64_t itt) {
  Dev d = c->dev();
  int mode = c->cfg.mode;
  bool linear = mode == SWM_MODE_LIN_REST || mode == SWM_MODE_LIN_MEAN;
  if (mode == SWM_MODE_NONLINEAR) LAUNCH(k_D_nonlinear, d);
  if (!linear || itt == 0) LAUNCH(k_D_interp, d);
  if (mode == SWM_MODE_NONLINEAR || mode == SWM_MODE_LIN_MEAN) LAUNCH(k_vorticity, d);
  if (mode != SWM_MODE_NONE) {
    LAUNCH(k_pot, d);
    LAUNCH(k_edens, d);
  }
  LAUNCH(k_massflux, d);
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// SWM_forcing_update (:135-170) or the constant part of SWM_forcing_init
// (:124-125).  Streams are visited in the reference's linked-list order: the
// head (first namelist record) first, then the others newest first
// (generic_list.f90:87-103 inserts after the head).
int plain_forcing_update(swm_gpu_ctx *c, int64_t itt, int constant_part) {
  Dev d = c->dev();
  if (!constant_part) LAUNCH(k_forcing_reset, d);
  int ns = (int)c->streams.size();
  if (ns == 0) {
    SWM_CK(cudaGetLastError());
    return SWM_GPU_OK;
  }
  std::vector<int> order;
  order.push_back(0);
  for (int s = ns - 1; s >= 1; s--) order.push_back(s);
  for (int q : order) {
    const Stream &s = c->streams[q];
    bool tdf = !s.is_const;
    if (constant_part == (int)tdf) continue;  // process when isTDF != isConstant
    double *Fx = s.is_const ? d.Fxc : d.Fx, *Fy = s.is_const ? d.Fyc : d.Fy, *Fe = s.is_const ? d.Fec : d.Fe;
    double r = 0., im = 0.;
    if (s.type == SWM_FRC_OSC) {
      r = cos(s.omega * (double)itt * c->cfg.dt);
      im = sin(s.omega * (double)itt * c->cfg.dt);
    }
    LAUNCH(k_stream, d, s, Fx, Fy, Fe, r, im);
  }
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// the coefficient table of k_latmix_p for this Ah (formed on first use)
static int latp_table(swm_gpu_ctx *c, double Ah, const double **out) {
  for (int q = 0; q < 2; q++)
    if (c->latp[q] && c->latp_ah[q] == Ah) {
      *out = c->latp[q];
      return SWM_GPU_OK;
    }
  const int q = c->latp[0] ? 1 : 0;
  SWM_REQUIRE(!c->latp[q], "lateral mixing: more than two mixing coefficients");
  SWM_CK(cudaMalloc((void **)&c->latp[q], (size_t)LATP_N * c->ny * sizeof(double)));
  c->latp_ah[q] = Ah;
  k_latmix_tab_p<<<(c->ny + 127) / 128, 128, 0, c->stream>>>(c->dev(), Ah, c->latp[q]);
  c->launches++;
  SWM_CK(cudaGetLastError());
  *out = c->latp[q];
  return SWM_GPU_OK;
}

static int latuv_table(swm_gpu_ctx *c, const double **out) {
  if (!c->latuv) {
    SWM_CK(cudaMalloc((void **)&c->latuv, (size_t)LATUV_N * c->ny * sizeof(double)));
    k_latmix_tab_uv<<<(c->ny + 127) / 128, 128, 0, c->stream>>>(c->dev(), c->latuv);
    c->launches++;
    SWM_CK(cudaGetLastError());
  }
  *out = c->latuv;
  return SWM_GPU_OK;
}

#define PTRY(x)                          \
  do {                                   \
    int rc_ = (x);                       \
    if (rc_ != SWM_GPU_OK) return rc_;   \
  } while (0)

// the coefficient tables the plain step needs, formed before a stream
// capture records steps (they are allocated on first use)
int plain_prepare(swm_gpu_ctx *c) {
  if (!c->pdiv_ready && !(c->impl[0] && c->impl[1] && c->impl[2])) {
    c->pdiv = false;  // no damping factors yet: the division operator
  } else if (!c->pdiv_ready) {
    const size_t n = c->n;
    if (!c->prow) SWM_CK(cudaMalloc((void **)&c->prow, (size_t)PROW_N * c->ny * sizeof(double)));
    for (int q = 0; q < 3; q++)
      if (!c->rimpl[q]) SWM_CK(cudaMalloc((void **)&c->rimpl[q], n * sizeof(double)));
    if (!c->pdiv_bad) SWM_CK(cudaMalloc((void **)&c->pdiv_bad, sizeof(int)));
    SWM_CK(cudaMemsetAsync(c->pdiv_bad, 0, sizeof(int), c->stream));
    const Dev d = c->dev();
    k_plain_rows<<<(c->ny + 127) / 128, 128, 0, c->stream>>>(d, c->prow, c->pdiv_bad);
    k_plain_rimpl<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(d, c->rimpl[0], c->rimpl[1], c->rimpl[2],
                                                                   c->pdiv_bad);
    c->launches += 2;
    SWM_CK(cudaGetLastError());
    int bad = 0;
    SWM_CK(cudaMemcpyAsync(&bad, c->pdiv_bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SWM_CK(cudaStreamSynchronize(c->stream));
    c->pdiv = !bad && div_host_range(c->hg.dLambda) && div_host_range(c->hg.dTheta) &&
              div_host_range(c->cfg.A * c->hg.dTheta);
    c->pdiv_ready = true;
  }
  if (!c->cfg.lateral_mixing) return SWM_GPU_OK;
  const double *t = nullptr;
  PTRY(latuv_table(c, &t));
  if (c->cfg.mixing_kind == SWM_MIX_BIHARMONIC) {
    PTRY(latp_table(c, 1., &t));
    return latp_table(c, -c->cfg.bih, &t);
  }
  return latp_table(c, c->cfg.Ah, &t);
}

// SWM_timestep_step (swm_nonlinear_timestep_module.f90:164-180)
int plain_step(swm_gpu_ctx *c, int64_t itt) {
  PTRY(plain_prepare(c));
  Dev d = c->dev();
  if (c->cfg.lateral_mixing) {
    const double *tuv = nullptr, *tp = nullptr;
    PTRY(latuv_table(c, &tuv));
    if (c->cfg.mixing_kind == SWM_MIX_BIHARMONIC) {
      // project extension: Laplacian-type operator with unit thickness and
      // Ah = 1, then the thickness-weighted operator with Ah = -bih
      const double *t1 = nullptr;
      PTRY(latp_table(c, 1., &t1));
      PTRY(latp_table(c, -c->cfg.bih, &tp));
      LAUNCH(k_latmix_p, d, t1, d.u0, d.v0, c->ones, c->ones, c->bh[0], c->bh[1]);
      LAUNCH(k_latmix_uv, d, tuv, c->bh[0], c->bh[1], c->ones, c->ones, c->bh[2], c->bh[3], 1);
      LAUNCH(k_latmix_p, d, tp, c->bh[2], c->bh[3], d.D, d.Dh, d.pll, d.plt);
    } else {
      PTRY(latp_table(c, c->cfg.Ah, &tp));
      LAUNCH(k_latmix_p, d, tp, d.u0, d.v0, d.D, d.Dh, d.pll, d.plt);
    }
    LAUNCH(k_latmix_uv, d, tuv, d.pll, d.plt, d.Du, d.Dv, d.lmu, d.lmv, 0);
  }
  LAUNCH(k_tend_eta, d);
  LAUNCH(k_tend_u, d);
  LAUNCH(k_tend_v, d);
  ABCoef ab;
  ab.tstep = (int)(itt < 3 ? itt : 3);
  const double chi = c->cfg.ab_chi;
  double tab[4][3] = {{0, 0, 0}, {1., 0, 0}, {-0.5 - chi, 1.5 + chi, 0}, {5. / 12., -16. / 12., 23. / 12.}};
  for (int q = 0; q < 3; q++) {
    ab.c[q] = tab[ab.tstep][q];
    ab.dtc[q] = c->cfg.dt * ab.c[q];
  }
  LAUNCH(k_integrate, d, ab);
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

}  // namespace swm
