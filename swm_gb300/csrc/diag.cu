// diag.cu -- diagnostics on the device.
//
// computeStreamfunction (calc_lib.f90:727-780): psi on the H grid from the
// zonal sums of v along rows and the meridional sums of u along columns,
// [times the face depths when BAROTROPIC].  Every SUM of the reference runs
// in its own order (a suffix along a row summed from its west end, a prefix
// along a column summed from the south), and this file is compiled without
// FMA contraction, so psi is bit for bit the FP64 restatement's.
//
// Time averages of diagTask (diagTask.f90:266-338): buffer = buffer + dT *
// field (or field^2), count = count + dT, mean = buffer / count, kept in
// FP64 on the device so an averaging task reads back one field per period.
#include <vector>
#include "ctx.h"

namespace swm {

struct PsiArgs {
  int nx, ny, bt;
  double A, dL, dT;
  const double *u, *v, *Hu, *Hv, *cV;
  const int8_t *oU, *oV;
  double *psi, *s1;
};

// row 0: psi(i, 1) = -sum_{q=i}^{Nx-1} [H_v] ocean_v v * A cos dLambda
__global__ void k_psi_row0(PsiArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nx - 1) return;
  double s = 0.;
  for (int q = i; q <= a.nx - 2; q++) s = s + (a.bt ? a.Hv[q] * a.oV[q] * a.v[q] : a.oV[q] * a.v[q]);
  a.psi[i] = (-1) * s * a.A * a.cV[0] * a.dL;
}

// column Nx: psi(Nx, j) = -sum_{q<j} [H_u] ocean_u u * A dTheta (one
// thread: the running sum adds the terms in the reference's order)
__global__ void k_psi_col(PsiArgs a) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s = 0.;
  for (int j = 1; j < a.ny; j++) {
    const size_t k = (a.nx - 1) + (size_t)a.nx * (j - 1);
    s = s + (a.bt ? a.Hu[k] * a.oU[k] * a.u[k] : a.oU[k] * a.u[k]);
    a.psi[(a.nx - 1) + (size_t)a.nx * j] = (-1) * s * a.A * a.dT;
  }
}

// zonal suffix sums of the interior rows
__global__ void k_psi_s1(PsiArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nx - 1) return;
  for (int j = blockIdx.y + 1; j < a.ny; j += gridDim.y) {
    const double *v = a.v + (size_t)a.nx * j, *Hv = a.Hv + (size_t)a.nx * j;
    double s = 0.;
    for (int q = i; q <= a.nx - 2; q++) s = s + (a.bt ? Hv[q] * v[q] : v[q]);
    a.s1[i + (size_t)a.nx * j] = s;
  }
}

// one thread per column: meridional prefix sum and the mean of the two paths
__global__ void k_psi_combine(PsiArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nx - 1) return;
  double s2 = 0.;
  for (int j = 1; j < a.ny; j++) {
    const size_t kq = i + (size_t)a.nx * (j - 1), k = i + (size_t)a.nx * j;
    s2 = s2 + (a.bt ? a.Hu[kq] * a.u[kq] : a.u[kq]);
    a.psi[k] = ((-1) * a.s1[k] * a.A * a.cV[j] * a.dL + a.psi[(a.nx - 1) + (size_t)a.nx * j] - s2 * a.A * a.dT +
                a.psi[i]) / 2.;
  }
}

__global__ void k_diag_acc(double *buf, const double *f, size_t n, double w, int square) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) buf[k] = buf[k] + w * (square ? f[k] * f[k] : f[k]);
}

__global__ void k_diag_mean(double *buf, double *out, size_t n, double count) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    out[k] = buf[k] / count;
    buf[k] = 0.;
  }
}

// psi of the device state into c->psi (allocated on first use)
int device_streamfunction(swm_gpu_ctx *c) {
  const size_t n = c->n;
  if (!c->psi) {
    SWM_CK(cudaMalloc((void **)&c->psi, n * 8));
    SWM_CK(cudaMalloc((void **)&c->psi_tmp, n * 8));
  }
  Dev d = c->dev();
  PsiArgs a;
  a.nx = c->nx; a.ny = c->ny; a.bt = c->cfg.barotropic;
  a.A = c->cfg.A; a.dL = c->hg.dLambda; a.dT = c->hg.dTheta;
  a.u = d.u0; a.v = d.v0; a.Hu = c->d_H[GU]; a.Hv = c->d_H[GV]; a.cV = c->d_cos[GV];
  a.oU = c->d_ocean[GU]; a.oV = c->d_ocean[GV];
  a.psi = c->psi; a.s1 = c->psi_tmp;
  SWM_CK(cudaMemsetAsync(c->psi, 0, n * 8, c->stream));
  const unsigned bx = (unsigned)((c->nx + 127) / 128);
  k_psi_row0<<<bx, 128, 0, c->stream>>>(a);
  k_psi_col<<<1, 32, 0, c->stream>>>(a);
  if (c->ny > 1) {
    k_psi_s1<<<dim3(bx, c->ny - 1 < 65535 ? c->ny - 1 : 65535), 128, 0, c->stream>>>(a);
    k_psi_combine<<<bx, 128, 0, c->stream>>>(a);
  }
  c->launches += 4;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

int diag_accumulate(swm_gpu_ctx *c, int slot, const double *f, int square, double w) {
  if ((int)c->diag.size() <= slot) c->diag.resize(slot + 1);
  DiagAcc &a = c->diag[slot];
  if (!a.buf) {
    SWM_CK(cudaMalloc((void **)&a.buf, c->n * 8));
    SWM_CK(cudaMemsetAsync(a.buf, 0, c->n * 8, c->stream));
    a.count = 0.;
  }
  k_diag_acc<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(a.buf, f, c->n, w, square);
  c->launches++;
  a.count = a.count + w;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

int diag_mean(swm_gpu_ctx *c, int slot, double *dev_out, double *count) {
  SWM_REQUIRE(slot >= 0 && slot < (int)c->diag.size() && c->diag[slot].buf, "swm_gpu_diag_mean: empty slot");
  DiagAcc &a = c->diag[slot];
  SWM_REQUIRE(a.count != 0., "swm_gpu_diag_mean: nothing accumulated");
  k_diag_mean<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(a.buf, dev_out, c->n, a.count);
  c->launches++;
  if (count) *count = a.count;
  a.count = 0.;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// getChunkData (memchunk_module.f90:214-246) on the device: the record at
// the bracket's lower end, or y0 + (t - t0) (y1 - y0) / (t1 - t0) between two
// records (r1 < 0: exactly record r0), in the restatement's operation order
__global__ void k_stream_interp(const double *rec, double *dst, size_t n, int r0, int r1, double t, double t0,
                                double t1) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double y0 = rec[(size_t)r0 * n + k];
  if (r1 < 0) {
    dst[k] = y0;
    return;
  }
  const double y1 = rec[(size_t)r1 * n + k];
  dst[k] = y0 + (t - t0) * (y1 - y0) / (t1 - t0);
}

int stream_interp(swm_gpu_ctx *c, const double *rec, double *dst, int r0, int r1, double t, double t0, double t1) {
  k_stream_interp<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(rec, dst, c->n, r0, r1, t, t0, t1);
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

void diag_free(swm_gpu_ctx *c) {
  for (auto &a : c->diag) cudaFree(a.buf);
  c->diag.clear();
  cudaFree(c->psi);
  cudaFree(c->psi_tmp);
  c->psi = c->psi_tmp = nullptr;
}

}  // namespace swm
