// tracer.cu -- passive tracers (tracer_module.f90, tracer_vars.f90), FP64,
// one kernel per reference loop nest; compiled with -fmad=false like plain.cu.
#include "ctx.h"

namespace swm {

__device__ __forceinline__ int tip1(int i, int n) { return i + 1 == n ? 0 : i + 1; }
__device__ __forceinline__ int tim1(int i, int n) { return i == 0 ? n - 1 : i - 1; }

// TRC_initCoeffs (tracer_module.f90:291-342); coefficient c of cell k at
// coeff[c * n + k] (structure of arrays).  guard = 1 replaces the 0/0 of
// land-land pairs by 0 (the reference produces NaN there).
__global__ void k_trc_coeff(Dev d, double *coeff, int guard) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  size_t n = (size_t)d.nx * d.ny, k = i + (size_t)d.nx * j;
  int ip = tip1(i, d.nx), im = tim1(i, d.nx), jp = tip1(j, d.ny), jm = tim1(j, d.ny);
  const int8_t *oE = d.ocean[GE], *oU = d.ocean[GU], *oV = d.ocean[GV];
  size_t kip = ip + (size_t)d.nx * j, kim = im + (size_t)d.nx * j;
  size_t kjp = i + (size_t)d.nx * jp, kjm = i + (size_t)d.nx * jm;
  double o0 = oE[k], oip = oE[kip], oim = oE[kim], ojp = oE[kjp], ojm = oE[kjm];
  double A = d.A, dL = d.dLambda, dT = d.dTheta;
  const double *cu = d.cosl[GU], *cv = d.cosl[GV], *ce = d.cosl[GE];
#define GD(den) ((guard && (den) == 0.) ? 1. : (den))
  coeff[0 * n + k] = -1. * oU[kip] * oip / GD(oip + o0) / A / dL / ce[j];
  coeff[1 * n + k] = 1. * oU[k] * oim / GD(oim + o0) / A / dL / ce[j];
  coeff[2 * n + k] = -1. * oV[kjp] * cv[jp] * ojp / GD(ojp + o0) / A / dT / ce[j];
  coeff[3 * n + k] = 1. * oV[k] * cv[j] * ojm / GD(ojm + o0) / A / dT / ce[j];
  coeff[4 * n + k] = -1. * oU[kip] * o0 / GD(oip + o0) / A / dL / ce[j];
  coeff[5 * n + k] = 1. * oU[k] * o0 / GD(oim + o0) / A / dL / ce[j];
  coeff[6 * n + k] = -1. * oV[kjp] * cv[jp] * o0 / GD(ojp + o0) / A / dT / ce[j];
  coeff[7 * n + k] = 1. * oV[k] * cv[j] * o0 / GD(ojm + o0) / A / dT / ce[j];
#undef GD
  coeff[8 * n + k] = 1. * oU[kip] / (dL * dL) / (A * A) / cu[j] / ce[j];
  coeff[9 * n + k] = -1. * oU[k] / (dL * dL) / (A * A) / cu[j] / ce[j];
  coeff[10 * n + k] = 1. * oV[kjp] * cv[jp] / (dT * dT) / (A * A) / ce[j];
  coeff[11 * n + k] = -1. * oV[k] * cv[j] / (dT * dT) / (A * A) / ce[j];
}

struct TrcView {
  double *CH0, *CH1, *G[3], *C, *C0, *gamma, *impl, *uhc, *vhc, *diff;
  double kappa_h;
};

// TRC_tracer_incr, diffusion loop (:169-180)
__global__ void k_trc_diff(Dev d, TrcView t, const double *coeff) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  size_t n = (size_t)d.nx * d.ny, k = i + (size_t)d.nx * j;
  if (d.ocean[GE][k] == 0) return;
  size_t ip = tip1(i, d.nx) + (size_t)d.nx * j, im = tim1(i, d.nx) + (size_t)d.nx * j;
  size_t jp = i + (size_t)d.nx * tip1(j, d.ny), jm = i + (size_t)d.nx * tim1(j, d.ny);
  const double *C = t.C, *hu = d.Du, *hv = d.Dv;
  double kap = t.kappa_h;
  t.diff[k] = kap * hu[ip] * (C[ip] - C[k]) * coeff[8 * n + k] + kap * hu[k] * (C[k] - C[im]) * coeff[9 * n + k] +
              kap * hv[jp] * (C[jp] - C[k]) * coeff[10 * n + k] + kap * hv[k] * (C[k] - C[jm]) * coeff[11 * n + k];
}

// Extension: third-order upwind-biased face value of CH between cells L and
// R (R east or north of L; Lm behind L, Rp beyond R) for face velocity vel;
// the reference's mask-weighted mean where one of the four cells is land
__device__ double ub3_face(const double *CH, const int8_t *oE, size_t Lm, size_t L, size_t R, size_t Rp,
                           double vel) {
  if (oE[Lm] && oE[L] && oE[R] && oE[Rp]) {
    if (vel >= 0.) return ((-1. * CH[Lm] + 5. * CH[L]) + 2. * CH[R]) / 6.;
    return ((2. * CH[L] + 5. * CH[R]) - 1. * CH[Rp]) / 6.;
  }
  double den = (double)(oE[L] + oE[R]);
  if (den == 0.) return 0.;
  return ((double)oE[L] * CH[L] + (double)oE[R] * CH[R]) / den;
}

__device__ double ub3_advection(const Dev &d, const double *CH, const double *u, const double *v, int i, int j) {
  const int8_t *oE = d.ocean[GE], *oU = d.ocean[GU], *oV = d.ocean[GV];
  const double *cv = d.cosl[GV], *ce = d.cosl[GE];
  const int nx = d.nx, ny = d.ny;
  const int ip = tip1(i, nx), im = tim1(i, nx), jp = tip1(j, ny), jm = tim1(j, ny);
  auto K = [nx](int a, int b) { return a + (size_t)nx * b; };
  size_t k = K(i, j);
  double fe = ub3_face(CH, oE, K(im, j), k, K(ip, j), K(tip1(ip, nx), j), u[K(ip, j)]);
  double fw = ub3_face(CH, oE, K(tim1(im, nx), j), K(im, j), k, K(ip, j), u[k]);
  double fn = ub3_face(CH, oE, K(i, jm), k, K(i, jp), K(i, tip1(jp, ny)), v[K(i, jp)]);
  double fs = ub3_face(CH, oE, K(i, tim1(jm, ny)), K(i, jm), k, K(i, jp), v[k]);
  double rdl = 1. / (d.A * d.dLambda * ce[j]), rdt = 1. / (d.A * d.dTheta * ce[j]);
  double ax = -1. * oU[K(ip, j)] * u[K(ip, j)] * fe + (double)oU[k] * u[k] * fw;
  double ay = -1. * oV[K(i, jp)] * cv[jp] * v[K(i, jp)] * fn + (double)oV[k] * cv[j] * v[k] * fs;
  return ax * rdl + ay * rdt;
}

// TRC_tracer_incr, forcing and increment loops (:182-207); the increment is
// written to slot 3 of the ring
__global__ void k_trc_incr(Dev d, TrcView t, const double *coeff, int flux) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  size_t n = (size_t)d.nx * d.ny, k = i + (size_t)d.nx * j;
  size_t ip = tip1(i, d.nx) + (size_t)d.nx * j, im = tim1(i, d.nx) + (size_t)d.nx * j;
  size_t jp = i + (size_t)d.nx * tip1(j, d.ny), jm = i + (size_t)d.nx * tim1(j, d.ny);
  const double *CH = t.CH0, *C = t.C, *u = d.u0, *v = d.v0;
  double forcing = C[k] * d.Fe[k];
  if (flux == 1) {
    t.G[2][k] = d.ocean[GE][k] ? (ub3_advection(d, CH, u, v, i, j) + t.diff[k] -
                                  t.gamma[k] * d.D[k] * (C[k] - t.C0[k]) + forcing)
                               : 0.;
    return;
  }
  const double *c = coeff;
  t.G[2][k] = (CH[ip] * u[ip] * c[0 * n + k] + CH[im] * u[k] * c[1 * n + k] + CH[jp] * v[jp] * c[2 * n + k] +
               CH[jm] * v[k] * c[3 * n + k] + CH[k] * u[ip] * c[4 * n + k] + CH[k] * u[k] * c[5 * n + k] +
               CH[k] * v[jp] * c[6 * n + k] + CH[k] * v[k] * c[7 * n + k] + t.diff[k] -
               t.gamma[k] * d.D[k] * (C[k] - t.C0[k]) + forcing);
}

// TRC_tracer_integrate (:216-232) -> integrate_AB_vec
__global__ void k_trc_integrate(Dev d, TrcView t, double c0, double c1, double c2, int tstep) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)d.nx * d.ny) return;
  double cc[3] = {c0, c1, c2};
  double a = t.CH0[k];
  for (int q = 0; q < tstep; q++) a = a + d.dt * cc[q] * t.G[q][k];
  t.CH1[k] = a / t.impl[k];
}

// TRC_tracer_advance, diagnostic part (:263-278)
__global__ void k_trc_C(Dev d, TrcView t, int guard) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)d.nx * d.ny) return;
  t.C[k] = (guard && d.D[k] == 0.) ? 0. : t.CH0[k] / d.D[k];  // guard: 0/0 on dry land -> 0
}
__global__ void k_trc_flux(Dev d, TrcView t) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  size_t k = i + (size_t)d.nx * j;
  size_t im = tim1(i, d.nx) + (size_t)d.nx * j, jm = i + (size_t)d.nx * tim1(j, d.ny);
  t.uhc[k] = d.mu[k] * .5 * (t.C[k] + t.C[im]);
  t.vhc[k] = d.mv[k] * .5 * (t.C[k] + t.C[jm]);
}

static TrcView view(const Tracer &T) {
  TrcView v;
  v.CH0 = T.CH[T.n0];
  v.CH1 = T.CH[1 - T.n0];
  for (int s = 0; s < 3; s++) v.G[s] = T.G[(T.g0 + s) % 3];
  v.C = T.C; v.C0 = T.C0; v.gamma = T.gamma; v.impl = T.impl;
  v.uhc = T.uhc; v.vhc = T.vhc; v.diff = T.diff;
  v.kappa_h = T.kappa_h;
  return v;
}

static dim3 tblk() { return dim3(32, 8); }
static dim3 tgrd(const swm_gpu_ctx *c) { return dim3((c->nx + 31) / 32, (c->ny + 7) / 8); }

int tracer_init_coeffs(swm_gpu_ctx *c) {
  if (!c->trc_coeff) SWM_CK(cudaMalloc((void **)&c->trc_coeff, 12 * c->n * sizeof(double)));
  k_trc_coeff<<<tgrd(c), tblk(), 0, c->stream>>>(c->dev(), c->trc_coeff, c->cfg.tracer_nan_guard);
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

int tracer_step(swm_gpu_ctx *c, int64_t itt) {
  Dev d = c->dev();
  int tstep = (int)(itt < 3 ? itt : 3);
  const double chi = c->cfg.ab_chi;
  double tab[4][3] = {{0, 0, 0}, {1., 0, 0}, {-0.5 - chi, 1.5 + chi, 0}, {5. / 12., -16. / 12., 23. / 12.}};
  unsigned nb = (unsigned)((c->n + 255) / 256);
  for (auto &T : c->tracers) {
    TrcView v = view(T);
    k_trc_diff<<<tgrd(c), tblk(), 0, c->stream>>>(d, v, c->trc_coeff);
    k_trc_incr<<<tgrd(c), tblk(), 0, c->stream>>>(d, v, c->trc_coeff, c->cfg.tracer_flux);
    k_trc_integrate<<<nb, 256, 0, c->stream>>>(d, v, tab[tstep][0], tab[tstep][1], tab[tstep][2], tstep);
    c->launches += 3;
  }
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

int tracer_advance(swm_gpu_ctx *c) {
  Dev d = c->dev();
  unsigned nb = (unsigned)((c->n + 255) / 256);
  for (auto &T : c->tracers) {
    T.g0 = (T.g0 + 1) % 3;
    T.n0 = 1 - T.n0;
    TrcView v = view(T);
    k_trc_C<<<nb, 256, 0, c->stream>>>(d, v, c->cfg.tracer_nan_guard);
    k_trc_flux<<<tgrd(c), tblk(), 0, c->stream>>>(d, v);
    c->launches += 2;
  }
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

}  // namespace swm

using namespace swm;

#define TRY_T(x)                         \
  do {                                   \
    int rc_ = (x);                       \
    if (rc_ != SWM_GPU_OK) return rc_;   \
  } while (0)

extern "C" {

int trc_gpu_add(swm_gpu_ctx *c, double kappa_h, double cons, double gamma_c, const double *C, const double *C0,
                const double *gfield, const double *cfield, int *id) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5, "trc_gpu_add: call after swm_gpu_initial_conditions");
  SWM_REQUIRE(c->tracers.size() < 16, "trc_gpu_add: too many tracers");
  size_t n = c->n;
  Tracer T;
  T.kappa_h = kappa_h;
  double **bufs[] = {&T.CH[0], &T.CH[1], &T.G[0], &T.G[1], &T.G[2], &T.C, &T.C0, &T.gamma, &T.impl, &T.uhc, &T.vhc, &T.diff};
  for (double **b : bufs) {
    SWM_CK(cudaMalloc((void **)b, n * sizeof(double)));
    SWM_CK(cudaMemsetAsync(*b, 0, n * sizeof(double), c->stream));
  }
  // TRC_add_to_list (tracer_vars.f90:152-161): CH = SWM_D * C, impl = 1 + dt*cons
  std::vector<double> Cv(n), C0v(n), gv(n), impl(n), D(n), CH(n);
  for (size_t k = 0; k < n; k++) {
    Cv[k] = C ? C[k] : 0.;
    C0v[k] = C0 ? C0[k] : 0.;
    gv[k] = gfield ? gfield[k] : gamma_c;
    impl[k] = 1. + c->cfg.dt * (cfield ? cfield[k] : cons);
  }
  Dev d = c->dev();
  if (c->cfg.path != SWM_PATH_PLAIN_FP64) {
    TRY_T(fused_sync_state(c));
    TRY_T(plain_diagnostics(c, 1));
  }
  SWM_CK(cudaMemcpyAsync(D.data(), d.D, n * 8, cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  for (size_t k = 0; k < n; k++) CH[k] = D[k] * Cv[k];
  SWM_CK(cudaMemcpy(T.CH[0], CH.data(), n * 8, cudaMemcpyHostToDevice));
  SWM_CK(cudaMemcpy(T.C, Cv.data(), n * 8, cudaMemcpyHostToDevice));
  SWM_CK(cudaMemcpy(T.C0, C0v.data(), n * 8, cudaMemcpyHostToDevice));
  SWM_CK(cudaMemcpy(T.gamma, gv.data(), n * 8, cudaMemcpyHostToDevice));
  SWM_CK(cudaMemcpy(T.impl, impl.data(), n * 8, cudaMemcpyHostToDevice));
  if (c->cfg.path == SWM_PATH_FUSED_FP32C) TRY_T(trc32_add(c, CH, C0v, gv, impl, kappa_h));
  c->tracers.push_back(T);
  if (id) *id = (int)c->tracers.size() - 1;
  return SWM_GPU_OK;
}

int trc_gpu_init(swm_gpu_ctx *c) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && !c->tracers.empty(), "trc_gpu_init: no tracer added");
  if (trc32_active(c)) return trc32_init(c);
  return tracer_init_coeffs(c);
}

int trc_gpu_get_field(swm_gpu_ctx *c, int t, int f, double *out) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && t >= 0 && t < (int)c->tracers.size() && out, "trc_gpu_get_field: bad arguments");
  const Tracer &T = c->tracers[t];
  if (trc32_active(c)) {
    // FP32 path: CH and C = CH / D are formed on request; the other fields
    // are not kept
    SWM_REQUIRE(f == TRC_F_CH || f == TRC_F_C, "trc_gpu_get_field: the FP32 tracer path keeps CH and C only");
    if (f == TRC_F_C && !c->cfg.frozen_flow) {
      TRY_T(fused_sync_state(c));
      TRY_T(plain_diagnostics(c, 1));
    }
    TRY_T(trc32_export(c, t, f == TRC_F_C, T.uhc));
    SWM_CK(cudaMemcpyAsync(out, T.uhc, c->n * 8, cudaMemcpyDeviceToHost, c->stream));
    SWM_CK(cudaStreamSynchronize(c->stream));
    return SWM_GPU_OK;
  }
  const double *p = nullptr;
  switch (f) {
    case TRC_F_CH: p = T.CH[T.n0]; break;
    case TRC_F_C: p = T.C; break;
    case TRC_F_G: p = T.G[(T.g0 + 1) % 3]; break;
    case TRC_F_UHC: p = T.uhc; break;
    case TRC_F_VHC: p = T.vhc; break;
    case TRC_F_DIFF: p = T.diff; break;
    case TRC_F_IMPL: p = T.impl; break;
  }
  SWM_REQUIRE(p, "trc_gpu_get_field: unknown field");
  SWM_CK(cudaMemcpyAsync(out, p, c->n * 8, cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}

}  // extern "C"
