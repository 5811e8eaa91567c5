// sor.cu -- red-black SOR of ElSolv_SOR.f90 on the GPU.
//
// Reference semantics: 5-point masked spherical Laplacian coefficients
// (init_ElSolv_SOR :54-62), colour 1 = i+j even (1-based) then colour 2,
// fixed Chebyshev relaxation schedule from rJacobi = 0.99999178 (binary32
// literal, :175, :206-210), stop on the first iteration whose correction norm
// sqrt(sum res^2) drops below eps (:213-218).  Each colour is one kernel; a
// finished solve turns the remaining kernels of a batch into no-ops through a
// device flag, so the host reads back once per batch instead of once per
// iteration.  The per-iteration norm is summed in a fixed order (per-block
// partials, then one block), so it is deterministic.
#include <cmath>
#include <vector>
#include "ctx.h"

struct SorState {
  double *c[5] = {};       // ElSolvSOR_c(:,:,1..5)
  double *chi = nullptr, *B = nullptr;
  double *partial = nullptr;   // per-block partial sums of res^2
  double *anorm2 = nullptr;    // running sum for the current iteration
  int *done = nullptr;         // [0] converged flag, [1] iteration at convergence
  double *anorm_hist = nullptr;
  double *und = nullptr, *vnd = nullptr;  // non-divergent flow
  int nblocks = 0;
};

namespace swm {

__global__ void k_sor_coeff(Dev d, SorState s) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  size_t k = i + (size_t)d.nx * j;
  int ip = i + 1 == d.nx ? 0 : i + 1, jp = j + 1 == d.ny ? 0 : j + 1;
  size_t ki = ip + (size_t)d.nx * j, kj = i + (size_t)d.nx * jp;
  const int8_t *oU = d.ocean[GU], *oV = d.ocean[GV];
  const double *cE = d.cosl[GE], *cV = d.cosl[GV];
  double A = d.A, dL = d.dLambda, dT = d.dTheta;
  double ax = (A * cE[j] * dL) * (A * cE[j] * dL);
  double ay = (A * A * cE[j] * (dT * dT));
  s.c[0][k] = oU[ki] / ax;
  s.c[1][k] = oU[k] / ax;
  s.c[2][k] = cV[jp] * oV[kj] / ay;
  s.c[3][k] = cV[j] * oV[k] / ay;
  s.c[4][k] = (-oU[ki] - oU[k]) / ax + (-cV[jp] * oV[kj] - cV[j] * oV[k]) / ay;
}

// one colour of one SOR iteration; colour 0 <-> (i+j) even in 0-based indices
__global__ void k_sor_colour(Dev d, SorState s, int colour, double relax) {
  __shared__ double red[256];
  int tid = threadIdx.y * blockDim.x + threadIdx.x;
  double r2 = 0.;
  if (!s.done[0]) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < d.nx && j < d.ny && ((i + j) & 1) == colour) {
      size_t k = i + (size_t)d.nx * j;
      if (d.ocean[GE][k] != 0) {
        int ip = i + 1 == d.nx ? 0 : i + 1, im = i == 0 ? d.nx - 1 : i - 1;
        int jp = j + 1 == d.ny ? 0 : j + 1, jm = j == 0 ? d.ny - 1 : j - 1;
        double *chi = s.chi;
        double res = relax * (s.c[0][k] * chi[ip + (size_t)d.nx * j] + s.c[1][k] * chi[im + (size_t)d.nx * j] +
                              s.c[2][k] * chi[i + (size_t)d.nx * jp] + s.c[3][k] * chi[i + (size_t)d.nx * jm] +
                              s.c[4][k] * chi[k] - s.B[k]) / s.c[4][k];
        chi[k] = chi[k] - res;
        r2 = res * res;
      }
    }
  }
  red[tid] = r2;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (tid < w) red[tid] += red[tid + w];
    __syncthreads();
  }
  if (tid == 0) s.partial[(size_t)colour * gridDim.x * gridDim.y + blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// sums both colours' partials in a fixed order and applies the stop test
__global__ void k_sor_check(SorState s, int nparts, int l, double eps) {
  __shared__ double red[256];
  if (s.done[0]) return;
  double acc = 0.;
  for (int q = threadIdx.x; q < 2 * nparts; q += blockDim.x) acc += s.partial[q];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double an = sqrt(red[0]);
    s.anorm_hist[0] = an;
    if (an < eps) {
      s.done[0] = 1;
      s.done[1] = l;
    }
  }
}

// computeDivergence (calc_lib.f90:607-622) of (u, v) onto the eta grid:
// pder_zonal(u, u_grid) + pder_meridional(cos_v v, v_grid) / cos_eta, with
// the mask tests of pder_zonal3D / pder_meridional3D (:892-998)
__global__ void k_sor_divergence(Dev d, const double *u, const double *v, double *div) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  size_t k = i + (size_t)d.nx * j;
  int ip = i + 1 == d.nx ? 0 : i + 1, jp = j + 1 == d.ny ? 0 : j + 1;
  size_t ki = ip + (size_t)d.nx * j, kj = i + (size_t)d.nx * jp;
  const int8_t *oU = d.ocean[GU], *oV = d.ocean[GV];
  const double bcE = d.ocean[GE][k] == 1 ? 1. : d.lbc;
  const double *cE = d.cosl[GE], *cV = d.cosl[GV];
  double dx = (oU[k] + oU[ki] == 0) ? 0. : bcE / (d.A * cE[j] * d.dLambda) * (u[ki] - u[k]);
  double dy = (oV[kj] + oV[k] == 0) ? 0. : bcE * (cV[jp] * v[kj] - cV[j] * v[k]) / (d.A * d.dTheta);
  div[k] = dx + dy / cE[j];
}

// computeGradient (:638-648) of chi on the eta grid (zonal part onto u,
// meridional onto v) subtracted from (u, v): computeNonDivergentFlowField
// (:548-590), u_nd = u - u_corr, v_nd = v - v_corr
__global__ void k_sor_nondiv(Dev d, const double *chi, const double *u, const double *v, double *u_nd,
                             double *v_nd) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  size_t k = i + (size_t)d.nx * j;
  int im = i == 0 ? d.nx - 1 : i - 1, jm = j == 0 ? d.ny - 1 : j - 1;
  size_t ki = im + (size_t)d.nx * j, kj = i + (size_t)d.nx * jm;
  const int8_t *oE = d.ocean[GE];
  const double bcU = d.ocean[GU][k] == 1 ? 1. : d.lbc, bcV = d.ocean[GV][k] == 1 ? 1. : d.lbc;
  double uc = (oE[ki] + oE[k] == 0) ? 0. : bcU / (d.A * d.cosl[GU][j] * d.dLambda) * (chi[k] - chi[ki]);
  double vc = (oE[kj] + oE[k] == 0) ? 0. : bcV * (chi[k] - chi[kj]) / (d.A * d.dTheta);
  u_nd[k] = u[k] - uc;
  v_nd[k] = v[k] - vc;
}

void sor_free(swm_gpu_ctx *c) {
  if (!c->sor) return;
  SorState *s = c->sor;
  for (int q = 0; q < 5; q++) cudaFree(s->c[q]);
  cudaFree(s->chi); cudaFree(s->B); cudaFree(s->partial); cudaFree(s->done); cudaFree(s->anorm_hist);
  cudaFree(s->und); cudaFree(s->vnd);
  delete s;
  c->sor = nullptr;
}

}  // namespace swm

using namespace swm;

extern "C" {

int elsolv_sor_gpu_init(swm_gpu_ctx *c) {
  SWM_REQUIRE(c && c->stage >= 1, "elsolv_sor_gpu_init: call after swm_gpu_domain");
  sor_free(c);
  SorState *s = new SorState();
  c->sor = s;
  size_t n = c->n;
  for (int q = 0; q < 5; q++) SWM_CK(cudaMalloc((void **)&s->c[q], n * 8));
  SWM_CK(cudaMalloc((void **)&s->chi, n * 8));
  SWM_CK(cudaMalloc((void **)&s->B, n * 8));
  dim3 b(32, 8), g((c->nx + 31) / 32, (c->ny + 7) / 8);
  s->nblocks = g.x * g.y;
  SWM_CK(cudaMalloc((void **)&s->partial, 2 * (size_t)s->nblocks * 8));
  SWM_CK(cudaMalloc((void **)&s->done, 2 * sizeof(int)));
  SWM_CK(cudaMalloc((void **)&s->anorm_hist, 8));
  SWM_CK(cudaMemsetAsync(s->chi, 0, n * 8, c->stream));  // calc_lib::chi starts at 0
  k_sor_coeff<<<g, b, 0, c->stream>>>(c->dev(), *s);
  c->launches++;
  SWM_CK(cudaGetLastError());
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}

}  // extern "C"

// main_ElSolv_SOR on the device arrays s->B (right-hand side) and s->chi
// (first guess in, solution out); returns SWM_GPU_ENOT_CONVERGED after
// max_count iterations
static int sor_solve_device(swm_gpu_ctx *c, double eps, int first_guess, int *iters, double *anorm) {
  SorState *s = c->sor;
  int mx = c->nx > c->ny ? c->nx : c->ny;
  int max_count = first_guess ? (int)lround(1000. * mx) : (int)lround(10. * mx);
  const double rJ = (double)(float)9.9999178e-1;
  SWM_CK(cudaMemsetAsync(s->done, 0, 2 * sizeof(int), c->stream));
  dim3 b(32, 8), g((c->nx + 31) / 32, (c->ny + 7) / 8);
  Dev d = c->dev();
  double relax = 1.;
  int done[2] = {0, 0};
  const int batch = 64;
  int l = 1;
  while (l <= max_count) {
    int lend = l + batch - 1 < max_count ? l + batch - 1 : max_count;
    for (; l <= lend; l++) {
      for (int oe = 1; oe <= 2; oe++) {
        // oe = 1: (i+j) even with 1-based indices = (i+j) even with 0-based
        k_sor_colour<<<g, b, 0, c->stream>>>(d, *s, oe == 1 ? 0 : 1, relax);
        c->launches++;
        if (oe == 1 && l == 1) relax = 1. / (1. - .5 * rJ * rJ);
        else relax = 1. / (1. - .25 * rJ * rJ * relax);
      }
      k_sor_check<<<1, 256, 0, c->stream>>>(*s, s->nblocks, l, eps);
      c->launches++;
    }
    SWM_CK(cudaGetLastError());
    SWM_CK(cudaMemcpyAsync(done, s->done, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SWM_CK(cudaStreamSynchronize(c->stream));
    if (done[0]) break;
  }
  double an = 0.;
  SWM_CK(cudaMemcpyAsync(&an, s->anorm_hist, 8, cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  if (anorm) *anorm = an;
  if (done[0]) {
    if (iters) *iters = done[1];
    return SWM_GPU_OK;
  }
  if (iters) *iters = max_count;
  set_error("elsolv_sor_gpu_solve: not converged after max_count iterations");
  return SWM_GPU_ENOT_CONVERGED;
}

extern "C" {

int elsolv_sor_gpu_solve(swm_gpu_ctx *c, const double *B, double *chi, double eps, int first_guess, int *iters,
                         double *anorm) {
  SWM_REQUIRE(c && c->sor && B && chi, "elsolv_sor_gpu_solve: call elsolv_sor_gpu_init first");
  SorState *s = c->sor;
  size_t n = c->n;
  SWM_CK(cudaMemcpyAsync(s->B, B, n * 8, cudaMemcpyHostToDevice, c->stream));
  SWM_CK(cudaMemcpyAsync(s->chi, chi, n * 8, cudaMemcpyHostToDevice, c->stream));
  int rc = sor_solve_device(c, eps, first_guess, iters, anorm);
  SWM_CK(cudaMemcpyAsync(chi, s->chi, n * 8, cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return rc;
}

// computeNonDivergentFlowField (calc_lib.f90:548-590) of the model's current
// (u, v): divergence, SOR for chi (chi kept on the device between calls as
// the reference keeps calc_lib::chi; first_guess as itt == 1), gradient,
// u_nd = u - grad_lambda chi, v_nd = v - grad_theta chi.  Outputs may be
// NULL.  SOR non-convergence is reported as by elsolv_sor_gpu_solve, with
// the non-divergent flow still formed.
int swm_gpu_nondivergent(swm_gpu_ctx *c, int first_guess, double eps, double *u_nd, double *v_nd, double *chi,
                         int *iters) {
  SWM_REQUIRE(c && c->stage >= 5 && c->sor, "swm_gpu_nondivergent: call elsolv_sor_gpu_init first");
  SorState *s = c->sor;
  const size_t n = c->n;
  if (!s->und) {
    SWM_CK(cudaMalloc((void **)&s->und, n * 8));
    SWM_CK(cudaMalloc((void **)&s->vnd, n * 8));
  }
  if (c->cfg.path != SWM_PATH_PLAIN_FP64 && c->fused) {
    int rc0 = fused_sync_state(c);
    if (rc0 != SWM_GPU_OK) return rc0;
  }
  Dev d = c->dev();
  dim3 b(32, 8), g((c->nx + 31) / 32, (c->ny + 7) / 8);
  k_sor_divergence<<<g, b, 0, c->stream>>>(d, d.u0, d.v0, s->B);
  c->launches++;
  SWM_CK(cudaGetLastError());
  int rc = sor_solve_device(c, eps, first_guess, iters, nullptr);
  if (rc != SWM_GPU_OK && rc != SWM_GPU_ENOT_CONVERGED) return rc;
  k_sor_nondiv<<<g, b, 0, c->stream>>>(d, s->chi, d.u0, d.v0, s->und, s->vnd);
  c->launches++;
  SWM_CK(cudaGetLastError());
  if (u_nd) SWM_CK(cudaMemcpyAsync(u_nd, s->und, n * 8, cudaMemcpyDeviceToHost, c->stream));
  if (v_nd) SWM_CK(cudaMemcpyAsync(v_nd, s->vnd, n * 8, cudaMemcpyDeviceToHost, c->stream));
  if (chi) SWM_CK(cudaMemcpyAsync(chi, s->chi, n * 8, cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return rc;
}

}  // extern "C"
