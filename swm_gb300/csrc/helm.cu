// helm.cu -- red-black SOR for the variable-coefficient Helmholtz problem
// div(H^-1 grad psi) - lambda psi = rhs (extension of ElSolv_SOR.f90, whose
// operator is the masked spherical Laplacian with a fixed Chebyshev
// relaxation schedule and an absolute stopping rule).
//
// Same sweep structure as main_ElSolv_SOR (:176-211): colour 0 then colour 1
// of (i + j), each point relaxed with the new values of the other colour.
// Face coefficients are formed on the fly from 1/H (mean of the two cells);
// land cells and the outer frame hold psi = 0.  Stopping: relative residual
// ||rhs - A psi||_2 / ||rhs||_2, checked every CHECK sweeps in FP64.
//
// Two solvers: FP64 sweeps (bit for bit with the FP64 restatement, this file
// is compiled without FMA contraction and the update's fused multiply-adds
// are explicit in both), and mixed precision: FP32 sweeps on
// the correction equation A e = r, with r = rhs - A psi formed in FP64 and
// psi += e accumulated in FP64 (iterative refinement).  An autotuner picks
// the relaxation factor in a given range from short trial solves and the
// thread-block shape of the sweep kernel from timings.
#include <cmath>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "ctx.h"

namespace swm {

constexpr int HELM_CHECK = 16;  // sweeps between residual checks
constexpr int HELM_RED = 1024;  // reduction blocks

// One FP32 SOR point update, shared by the global and the tiled kernels so
// both round alike: explicit fused multiply-adds, the diagonal applied as its
// reciprocal (formed once per cell)
__device__ __forceinline__ float sor32_update(float p, float r, float cxw, float cxe, float cys, float cyn, float rcc,
                                              float w, float e, float s, float n, float omega) {
  const float off = fmaf(cyn, n, fmaf(cys, s, fmaf(cxe, e, cxw * w)));
  const float gs = (r - off) * rcc;
  return fmaf(omega, gs - p, p);
}

__device__ __forceinline__ float face32(float a, float b, float rd2) { return (0.5f * (a + b)) * rd2; }


// FP64 coefficients formed once: west and south face coefficients and the
// reciprocal of the diagonal (the sweeps would otherwise be bound by the
// FP64 pipe, which forms them and divides at every point of every sweep)
__global__ void k_h_coeff64(int nx, int ny, const double *__restrict__ h, double rdx2, double rdy2, double lambda,
                            double *cx, double *cy, double *rcc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t k = (size_t)i + (size_t)nx * j;
  const double hk = h[k];
  const double cxw = i > 0 ? (0.5 * (hk + h[k - 1])) * rdx2 : 0.;
  const double cxe = i < nx - 1 ? (0.5 * (h[k + 1] + hk)) * rdx2 : 0.;
  const double cys = j > 0 ? (0.5 * (hk + h[k - nx])) * rdy2 : 0.;
  const double cyn = j < ny - 1 ? (0.5 * (h[k + nx] + hk)) * rdy2 : 0.;
  cx[k] = cxw;
  cy[k] = cys;
  rcc[k] = 1. / (-(((cxw + cxe) + cys) + cyn) - lambda);
}

// FP64 sweeps run on a colour-split layout: cell (i, j) of colour (i + j) % 2
// sits at j * W + i / 2 of its colour's arrays (W = ceil(nx / 2)) with its
// four face coefficients (0 at the frame), reciprocal diagonal, rhs and mask,
// so a colour pass reads only its own colour's arrays and the other
// colour's psi, contiguous, one thread per cell of the colour
struct Split64 {
  double *c[2][4];  // west, east, south, north face coefficients
  double *rcc[2], *rhs[2], *psi[2];
  uint8_t *mask[2];  // 0 also on the padding of rows with fewer cells
};

__global__ void k_h_split_coeff64(int nx, int ny, int W, const double *__restrict__ cx, const double *__restrict__ cy,
                                  const double *__restrict__ rcc, const int8_t *__restrict__ mask, Split64 s) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)nx * ny) return;
  const int i = (int)(k % nx), j = (int)(k / nx), col = (i + j) & 1;
  const size_t q = (size_t)j * W + (i >> 1);
  s.c[col][0][q] = cx[k];
  s.c[col][1][q] = i < nx - 1 ? cx[k + 1] : 0.;
  s.c[col][2][q] = cy[k];
  s.c[col][3][q] = j < ny - 1 ? cy[k + nx] : 0.;
  s.rcc[col][q] = rcc[k];
  s.mask[col][q] = mask[k] != 0;
}

// natural <-> colour-split copy of one field (join 0: natural -> split)
__global__ void k_h_split64(int nx, int ny, int W, double *nat, double *s0, double *s1, int join) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)nx * ny) return;
  const int i = (int)(k % nx), j = (int)(k / nx);
  double *sp = ((i + j) & 1) ? s1 : s0;
  const size_t q = (size_t)j * W + (i >> 1);
  if (join) nat[k] = sp[q];
  else sp[q] = nat[k];
}

// one colour of an FP64 sweep: off = cw w + ce e + cs s + cn n as nested
// fused multiply-adds, psi += omega ((rhs - off) / diag - psi) as one more
// (the arithmetic of orc_helmholtz_sor)
__global__ void k_h_sweep64(int nx, int ny, int W, Split64 s, int col, double omega) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)W * ny || !s.mask[col][q]) return;
  const int j = (int)(q / W), i = 2 * (int)(q - (size_t)j * W) + ((j + col) & 1);
  const double *P = s.psi[col ^ 1];
  const size_t r0 = (size_t)j * W;
  const double w = i > 0 ? P[r0 + ((i - 1) >> 1)] : 0., e = i < nx - 1 ? P[r0 + ((i + 1) >> 1)] : 0.;
  const double so = j > 0 ? P[r0 - W + (i >> 1)] : 0., n = j < ny - 1 ? P[r0 + W + (i >> 1)] : 0.;
  const double off =
      __fma_rn(s.c[col][0][q], w, __fma_rn(s.c[col][1][q], e, __fma_rn(s.c[col][2][q], so, s.c[col][3][q] * n)));
  const double gs = (s.rhs[col][q] - off) * s.rcc[col][q];
  double *x = s.psi[col];
  x[q] = __fma_rn(omega, gs - x[q], x[q]);
}

// one colour of an FP32 sweep over the whole grid (the arithmetic of k_h_tbr)
__global__ void k_h_sweep32(int nx, int ny, const float *__restrict__ h, const int8_t *__restrict__ mask,
                            const float *__restrict__ rhs, float *psi, float rdx2, float rdy2, float lambda,
                            float omega, int colour) {
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + ((j + colour) & 1);
  if (i >= nx || j >= ny) return;
  const size_t k = (size_t)i + (size_t)nx * j;
  if (!mask[k]) return;
  const float hk = h[k];
  const float cxw = i > 0 ? face32(hk, h[k - 1], rdx2) : 0.f;
  const float cxe = i < nx - 1 ? face32(h[k + 1], hk, rdx2) : 0.f;
  const float cys = j > 0 ? face32(hk, h[k - nx], rdy2) : 0.f;
  const float cyn = j < ny - 1 ? face32(h[k + nx], hk, rdy2) : 0.f;
  // the tiled kernel forms the next cell's west face as face32(h[k+1], h[k]),
  // this kernel forms this cell's east face the same way: same operand order
  const float rcc = 1.f / (-(((cxw + cxe) + cys) + cyn) - lambda);
  const float w = i > 0 ? psi[k - 1] : 0.f, e = i < nx - 1 ? psi[k + 1] : 0.f;
  const float s = j > 0 ? psi[k - nx] : 0.f, n = j < ny - 1 ? psi[k + nx] : 0.f;
  psi[k] = sor32_update(psi[k], rhs[k], cxw, cxe, cys, cyn, rcc, w, e, s, n, omega);
}

// K red-black sweeps of FP32 SOR on a region of 64 columns by YM rows
// (interior 64 - 4K by YM - 4K, halo 2K), each thread owning, for the whole
// launch, the cell pair of region columns 2tx (cell a) and 2tx + 1 (cell b)
// in rows ty + Ym.  A pair's face coefficients, reciprocal diagonals and rhs
// are formed once per launch and kept in registers (the pair shares its
// inner face).  psi is kept in shared memory split by column parity, so a
// warp's accesses are contiguous, and each cell's inner neighbour is the
// thread's own register.  Every neighbour of a cell has the other colour, so
// a pass reads only what the previous passes wrote.  Halo cells are relaxed
// with the arithmetic of the global sweep (sor32_update, same coefficients),
// so after 2K passes the interior equals K global sweeps bit for bit; rows
// that can no longer reach the interior are skipped.  Cells outside the grid
// hold psi = 0 and are never relaxed.
// TBR_Y x 32 threads per block, TBR_M rows per thread (64 registers: 2
// blocks, 32 warps per SM); TBR_Y even, so a thread's cells a share one
// colour
constexpr int TBR_Y = 16, TBR_M = 3;
template <int K>
__global__ void __launch_bounds__(32 * TBR_Y, 2) k_h_tbr(int nx, int ny, const float *__restrict__ hin,
                                                  const int8_t *__restrict__ mask, const float *__restrict__ rhs,
                                                  const float *__restrict__ pin, float *__restrict__ pout, float rdx2,
                                                  float rdy2, float lambda, float omega) {
  constexpr int M = TBR_M, Y = TBR_Y, W = 2 * K, RY = Y * M, TX = 64 - 2 * W, TY = RY - 2 * W;
  __shared__ float sa[RY][32], sb[RY][32];  // psi of the even / odd region columns
  __shared__ float ha[RY][32], hb[RY][32];  // 1/H, read while forming the coefficients
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * TX - W, y0 = blockIdx.y * TY - W;
  const int gxa = x0 + 2 * tx, gxb = gxa + 1;
  float pa[M], pb[M], ra[M], rb[M];                       // psi and rhs of cells a and b
  float cwa[M], cm[M], ceb[M], csa[M], cna[M], csb[M], cnb[M];  // face coefficients (cm: a's east = b's west)
  float qa[M], qb[M];                                     // reciprocal diagonals
  unsigned relax = 0;                                     // bit 2m: cell a of row m is relaxed, 2m + 1: cell b
#pragma unroll
  for (int m = 0; m < M; m++) {
    const int ly = ty + Y * m, gy = y0 + ly;
    const bool iny = gy >= 0 && gy < ny;
    const bool ina = iny && gxa >= 0 && gxa < nx, inb = iny && gxb >= 0 && gxb < nx;
    const size_t ka = ina ? (size_t)gxa + (size_t)nx * gy : 0, kb = inb ? (size_t)gxb + (size_t)nx * gy : 0;
    pa[m] = ina ? pin[ka] : 0.f;
    pb[m] = inb ? pin[kb] : 0.f;
    ra[m] = ina ? rhs[ka] : 0.f;
    rb[m] = inb ? rhs[kb] : 0.f;
    ha[ly][tx] = ina ? hin[ka] : 1.f;
    hb[ly][tx] = inb ? hin[kb] : 1.f;
    sa[ly][tx] = pa[m];
    sb[ly][tx] = pb[m];
    // the region's outer ring is never relaxed (its neighbours lie outside)
    const bool inner = ly >= 1 && ly < RY - 1;
    if (inner && ina && tx > 0 && mask[ka]) relax |= 1u << (2 * m);
    if (inner && inb && tx < 31 && mask[kb]) relax |= 2u << (2 * m);
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < M; m++) {
    const int ly = ty + Y * m, gy = y0 + ly;
    cwa[m] = cm[m] = ceb[m] = csa[m] = cna[m] = csb[m] = cnb[m] = qa[m] = qb[m] = 0.f;
    const bool da = (relax >> (2 * m)) & 1, db = (relax >> (2 * m + 1)) & 1;
    const float hka = ha[ly][tx], hkb = hb[ly][tx];
    if (da || db) cm[m] = gxa < nx - 1 && gxb > 0 ? face32(hkb, hka, rdx2) : 0.f;
    if (da) {
      cwa[m] = gxa > 0 ? face32(hka, hb[ly][tx - 1], rdx2) : 0.f;
      csa[m] = gy > 0 ? face32(hka, ha[ly - 1][tx], rdy2) : 0.f;
      cna[m] = gy < ny - 1 ? face32(ha[ly + 1][tx], hka, rdy2) : 0.f;
      qa[m] = 1.f / (-(((cwa[m] + cm[m]) + csa[m]) + cna[m]) - lambda);
    }
    if (db) {
      ceb[m] = gxb < nx - 1 ? face32(ha[ly][tx + 1], hkb, rdx2) : 0.f;
      csb[m] = gy > 0 ? face32(hkb, hb[ly - 1][tx], rdy2) : 0.f;
      cnb[m] = gy < ny - 1 ? face32(hb[ly + 1][tx], hkb, rdy2) : 0.f;
      qb[m] = 1.f / (-(((cm[m] + ceb[m]) + csb[m]) + cnb[m]) - lambda);
    }
  }
  // colour of this thread's cells a ((gx + gy) & 1, the same in all its rows)
  const int ca = (x0 + y0 + ty) & 1;
  // flat views: the ring columns' outer neighbours (never used: those cells
  // are not relaxed) then stay inside the arrays
  const float *fa = &sa[0][0], *fb = &sb[0][0];
#pragma unroll
  for (int pass = 0; pass < 2 * K; pass++) {
    const int lo = pass + 1, hi = RY - pass - 1;  // rows that still reach the interior
    const bool do_a = ca == (pass & 1);           // warp-uniform
#pragma unroll
    for (int m = 0; m < M; m++) {
      const int ly = ty + Y * m, l = ly * 32 + tx;
      // rows Ym .. Ym + Y - 1 lie in [lo, hi) in every pass unless m is the
      // first or last row group: only those test the row (warp-uniform)
      const bool mid = Y * m >= 2 * K && Y * m + Y <= RY - 2 * K;
      if (!mid && (ly < lo || ly >= hi)) continue;
      // relaxed as in the global sweep; cells not relaxed (land, outside the
      // grid, the region's ring) store their value back unchanged
      if (do_a) {
        const float v = sor32_update(pa[m], ra[m], cwa[m], cm[m], csa[m], cna[m], qa[m], fb[l - 1], pb[m],
                                     fa[l - 32], fa[l + 32], omega);
        pa[m] = ((relax >> (2 * m)) & 1) ? v : pa[m];
        sa[ly][tx] = pa[m];
      } else {
        const float v = sor32_update(pb[m], rb[m], cm[m], ceb[m], csb[m], cnb[m], qb[m], pa[m], fa[l + 1],
                                     fb[l - 32], fb[l + 32], omega);
        pb[m] = ((relax >> (2 * m + 1)) & 1) ? v : pb[m];
        sb[ly][tx] = pb[m];
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int m = 0; m < M; m++) {
    const int ly = ty + Y * m, gy = y0 + ly;
    if (ly < W || ly >= RY - W || gy >= ny) continue;
    if (2 * tx >= W && 2 * tx < 64 - W && gxa < nx) pout[(size_t)gxa + (size_t)nx * gy] = pa[m];
    if (2 * tx + 1 >= W && 2 * tx + 1 < 64 - W && gxb < nx) pout[(size_t)gxb + (size_t)nx * gy] = pb[m];
  }
}

// r = rhs - A psi on ocean cells (0 elsewhere) from the FP64 face
// coefficients, for an FP64 or FP32 iterate; per-block partial sums of r^2
template <typename T>
__global__ void k_h_resid_c(int nx, int ny, const double *__restrict__ cx, const double *__restrict__ cy,
                            double lambda, const int8_t *__restrict__ mask, const T *__restrict__ rhs,
                            const T *__restrict__ psi, double *r, double *partial) {
  __shared__ double red[256];
  double acc = 0.;
  const size_t n = (size_t)nx * ny;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    double rr = 0.;
    if (mask[k]) {
      const double cxw = cx[k], cxe = i < nx - 1 ? cx[k + 1] : 0., cys = cy[k], cyn = j < ny - 1 ? cy[k + nx] : 0.;
      const double cc = -(((cxw + cxe) + cys) + cyn) - lambda;
      const double w = i > 0 ? (double)psi[k - 1] : 0., e = i < nx - 1 ? (double)psi[k + 1] : 0.;
      const double s = j > 0 ? (double)psi[k - nx] : 0., nn = j < ny - 1 ? (double)psi[k + nx] : 0.;
      rr = (double)rhs[k] - (cxw * w + cxe * e + cys * s + cyn * nn + cc * (double)psi[k]);
    }
    if (r) r[k] = rr;
    acc += rr * rr;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_h_sumsq(const double *x, const int8_t *mask, size_t n, double *partial) {
  __shared__ double red[256];
  double acc = 0.;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    if (mask[k]) acc += x[k] * x[k];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_h_final(const double *partial, int nb, double *out) {
  __shared__ double red[256];
  double a = 0.;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) a += partial[b];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

__global__ void k_h_to32(const double *r, float *r32, float *e32, size_t n, double inv_scale) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    r32[k] = (float)(r[k] * inv_scale);
    e32[k] = 0.f;
  }
}

__global__ void k_h_axpy(double *psi, const float *e32, size_t n, double scale) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) psi[k] = psi[k] + scale * (double)e32[k];
}

}  // namespace swm

struct swm_helm {
  int device = -1;  // the CUDA device the solver was created on
  double *cx = nullptr, *cy = nullptr, *rcc = nullptr;  // FP64 coefficients
  swm::Split64 s64 = {};  // the FP64 sweeps' colour-split arrays (first FP64 solve)
  bool has_s64 = false;
  int W = 0;              // cells of a colour-split row
  int nx = 0, ny = 0;
  size_t n = 0;
  double dx = 0, dy = 0, lambda = 0;
  cudaStream_t stream = nullptr;
  double *hinv = nullptr, *psi = nullptr, *rhs = nullptr, *r = nullptr, *partial = nullptr, *out = nullptr;
  double *host = nullptr;  // pinned, 1 double
  float *hinv32 = nullptr, *e32 = nullptr, *r32 = nullptr, *e32b = nullptr;  // e32b: ping-pong of e32
  int tbk = 4;  // sweeps per temporally blocked FP32 launch
  int8_t *mask = nullptr;
  dim3 blk = dim3(64, 4);
  int64_t launches = 0;
};

namespace {
using namespace swm;

#define HTRY(x)                          \
  do {                                   \
    int rc_ = (x);                       \
    if (rc_ != SWM_GPU_OK) return rc_;   \
  } while (0)

dim3 sweep_grid(const swm_helm *h, dim3 b) {
  return dim3((unsigned)(((h->nx + 1) / 2 + b.x - 1) / b.x), (unsigned)((h->ny + b.y - 1) / b.y));
}

void sweep64(swm_helm *h, double omega) {
  const unsigned g = (unsigned)(((size_t)h->W * h->ny + 255) / 256);
  for (int colour = 0; colour < 2; colour++)
    k_h_sweep64<<<g, 256, 0, h->stream>>>(h->nx, h->ny, h->W, h->s64, colour, omega);
  h->launches += 2;
}

// the colour-split arrays of the FP64 sweeps, set up at the first FP64 solve
int split64_setup(swm_helm *h) {
  if (h->has_s64) return SWM_GPU_OK;
  h->W = (h->nx + 1) / 2;
  const size_t ns = (size_t)h->W * h->ny;
  Split64 &s = h->s64;
  for (int col = 0; col < 2; col++) {
    for (int f = 0; f < 4; f++) SWM_CK(cudaMalloc((void **)&s.c[col][f], ns * 8));
    SWM_CK(cudaMalloc((void **)&s.rcc[col], ns * 8));
    SWM_CK(cudaMalloc((void **)&s.rhs[col], ns * 8));
    SWM_CK(cudaMalloc((void **)&s.psi[col], ns * 8));
    SWM_CK(cudaMalloc((void **)&s.mask[col], ns));
    SWM_CK(cudaMemsetAsync(s.mask[col], 0, ns, h->stream));
  }
  h->has_s64 = true;
  const unsigned nb = (unsigned)((h->n + 255) / 256);
  k_h_split_coeff64<<<nb, 256, 0, h->stream>>>(h->nx, h->ny, h->W, h->cx, h->cy, h->rcc, h->mask, s);
  h->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// one field between the natural layout and the FP64 sweeps' split layout
void split64_field(swm_helm *h, double *nat, double *const *sp, int join) {
  const unsigned nb = (unsigned)((h->n + 255) / 256);
  k_h_split64<<<nb, 256, 0, h->stream>>>(h->nx, h->ny, h->W, nat, sp[0], sp[1], join);
  h->launches++;
}

void sweep32(swm_helm *h, float omega, dim3 b) {
  const dim3 g = sweep_grid(h, b);
  const float rdx2 = (float)(1. / (h->dx * h->dx)), rdy2 = (float)(1. / (h->dy * h->dy)), lam = (float)h->lambda;
  for (int colour = 0; colour < 2; colour++)
    k_h_sweep32<<<g, b, 0, h->stream>>>(h->nx, h->ny, h->hinv32, h->mask, h->r32, h->e32, rdx2, rdy2, lam, omega,
                                        colour);
  h->launches += 2;
}

template <int K>
void launch_tb32(swm_helm *h, float omega) {
  constexpr int TX = 64 - 4 * K, TY = TBR_Y * TBR_M - 4 * K;
  const dim3 g((h->nx + TX - 1) / TX, (h->ny + TY - 1) / TY), b(32, TBR_Y);
  const float rdx2 = (float)(1. / (h->dx * h->dx)), rdy2 = (float)(1. / (h->dy * h->dy)), lam = (float)h->lambda;
  k_h_tbr<K><<<g, b, 0, h->stream>>>(h->nx, h->ny, h->hinv32, h->mask, h->r32, h->e32, h->e32b, rdx2, rdy2, lam,
                                     omega);
}

// whole temporally blocked launches in n sweeps (none when tbk is 0: global
// sweeps only)
int tb_part(const swm_helm *h, int n) { return h->tbk > 0 ? n - n % h->tbk : 0; }

// n FP32 sweeps (a multiple of h->tbk) on A e = r32, ping-ponging e32/e32b;
// the result ends in h->e32
void sweeps_tb32(swm_helm *h, float omega, int n) {
  for (int s = 0; s < n && h->tbk > 0; s += h->tbk) {
    if (h->tbk == 4) launch_tb32<4>(h, omega);
    else if (h->tbk == 3) launch_tb32<3>(h, omega);
    else if (h->tbk == 2) launch_tb32<2>(h, omega);
    else launch_tb32<1>(h, omega);
    std::swap(h->e32, h->e32b);
    h->launches++;
  }
}

// ||rhs - A psi||^2 (FP64 accumulation); r written when wanted
template <typename T>
int resid2(swm_helm *h, const T *hh, const T *rhs, const T *psi, double *r, double *out) {
  (void)hh;
  k_h_resid_c<T><<<HELM_RED, 256, 0, h->stream>>>(h->nx, h->ny, h->cx, h->cy, h->lambda, h->mask, rhs, psi, r,
                                                  h->partial);
  k_h_final<<<1, 256, 0, h->stream>>>(h->partial, HELM_RED, h->out);
  h->launches += 2;
  SWM_CK(cudaGetLastError());
  SWM_CK(cudaMemcpyAsync(h->host, h->out, 8, cudaMemcpyDeviceToHost, h->stream));
  SWM_CK(cudaStreamSynchronize(h->stream));
  *out = h->host[0];
  return SWM_GPU_OK;
}

int rhs_norm(swm_helm *h, double *bn) {
  k_h_sumsq<<<HELM_RED, 256, 0, h->stream>>>(h->rhs, h->mask, h->n, h->partial);
  k_h_final<<<1, 256, 0, h->stream>>>(h->partial, HELM_RED, h->out);
  h->launches += 2;
  SWM_CK(cudaGetLastError());
  SWM_CK(cudaMemcpyAsync(h->host, h->out, 8, cudaMemcpyDeviceToHost, h->stream));
  SWM_CK(cudaStreamSynchronize(h->stream));
  *bn = std::sqrt(h->host[0]);
  return SWM_GPU_OK;
}

// FP32 sweeps on A e = r32 from e = 0 until ||r32 - A e|| <= tol ||r32||,
// until binary32 rounding stops the progress (a check that gains less than
// STALL over the previous one), or max_sweeps; returns the sweeps done and
// the reached relative residual
constexpr double STALL = 0.7;
int inner32(swm_helm *h, float omega, double tol, int max_sweeps, int *sweeps, double *rel) {
  double rn2 = 0.;
  // ||r32||: residual of e = 0
  HTRY(resid2<float>(h, h->hinv32, h->r32, h->e32, nullptr, &rn2));
  const double rn = std::sqrt(rn2);
  int s = 0, checks = 0;
  double rr = 1., prev = 1.;
  while (s < max_sweeps) {
    // 2 * HELM_CHECK sweeps between checks of the correction equation
    int blk = std::min(2 * HELM_CHECK, max_sweeps - s);
    const int tb = tb_part(h, blk);
    sweeps_tb32(h, omega, tb);
    for (int q = tb; q < blk; q++) sweep32(h, omega, h->blk);
    s += blk;
    double e2 = 0.;
    HTRY(resid2<float>(h, h->hinv32, h->r32, h->e32, nullptr, &e2));
    rr = rn > 0 ? std::sqrt(e2) / rn : 0.;
    if (rr <= tol || (++checks >= 2 && rr > STALL * prev)) break;
    prev = rr;
  }
  *sweeps = s;
  *rel = rr;
  return SWM_GPU_OK;
}

void helm_free(swm_helm *h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->hinv); cudaFree(h->psi); cudaFree(h->rhs); cudaFree(h->r); cudaFree(h->partial); cudaFree(h->out);
  cudaFreeHost(h->host);
  cudaFree(h->hinv32); cudaFree(h->e32); cudaFree(h->r32); cudaFree(h->mask); cudaFree(h->e32b);
  cudaFree(h->cx); cudaFree(h->cy); cudaFree(h->rcc);
  for (int col = 0; col < 2; col++) {
    for (int f = 0; f < 4; f++) cudaFree(h->s64.c[col][f]);
    cudaFree(h->s64.rcc[col]); cudaFree(h->s64.rhs[col]); cudaFree(h->s64.psi[col]); cudaFree(h->s64.mask[col]);
  }
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

}  // namespace

extern "C" {

int swm_helm_create(int nx, int ny, double dx, double dy, double lambda, const double *H, const int8_t *ocean,
                    swm_helm **out) {
  SWM_REQUIRE(nx >= 3 && ny >= 3 && dx > 0 && dy > 0 && H && ocean && out, "swm_helm_create: bad arguments");
  *out = nullptr;
  swm_helm *h = new swm_helm();
  if (cudaGetDevice(&h->device) != cudaSuccess) h->device = -1;
  h->nx = nx; h->ny = ny; h->n = (size_t)nx * ny; h->dx = dx; h->dy = dy; h->lambda = lambda;
  const size_t n = h->n;
  std::vector<double> hinv(n);
  std::vector<float> hinv32(n);
  for (size_t k = 0; k < n; k++) {
    if (!(H[k] > 0.)) {
      helm_free(h);
      set_error("swm_helm_create: depth must be positive everywhere (land is given by the ocean mask)");
      return SWM_GPU_EINVAL;
    }
    hinv[k] = 1. / H[k];
    hinv32[k] = (float)hinv[k];
  }
  bool ok = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc((void **)&h->hinv, n * 8) == cudaSuccess && cudaMalloc((void **)&h->psi, n * 8) == cudaSuccess &&
            cudaMalloc((void **)&h->rhs, n * 8) == cudaSuccess && cudaMalloc((void **)&h->r, n * 8) == cudaSuccess &&
            cudaMalloc((void **)&h->partial, HELM_RED * 8) == cudaSuccess &&
            cudaMalloc((void **)&h->out, 8) == cudaSuccess && cudaMallocHost((void **)&h->host, 8) == cudaSuccess &&
            cudaMalloc((void **)&h->hinv32, n * 4) == cudaSuccess && cudaMalloc((void **)&h->e32, n * 4) == cudaSuccess &&
            cudaMalloc((void **)&h->r32, n * 4) == cudaSuccess && cudaMalloc((void **)&h->mask, n) == cudaSuccess &&
            cudaMalloc((void **)&h->e32b, n * 4) == cudaSuccess &&
            cudaMalloc((void **)&h->cx, n * 8) == cudaSuccess && cudaMalloc((void **)&h->cy, n * 8) == cudaSuccess &&
            cudaMalloc((void **)&h->rcc, n * 8) == cudaSuccess;
  if (!ok) {
    helm_free(h);
    set_error("swm_helm_create: device allocation failed");
    return SWM_GPU_ENOMEM;
  }
  SWM_CK(cudaMemcpyAsync(h->hinv, hinv.data(), n * 8, cudaMemcpyHostToDevice, h->stream));
  SWM_CK(cudaMemcpyAsync(h->hinv32, hinv32.data(), n * 4, cudaMemcpyHostToDevice, h->stream));
  SWM_CK(cudaMemcpyAsync(h->mask, ocean, n, cudaMemcpyHostToDevice, h->stream));
  dim3 b(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  k_h_coeff64<<<g, b, 0, h->stream>>>(nx, ny, h->hinv, 1. / (dx * dx), 1. / (dy * dy), lambda, h->cx, h->cy, h->rcc);
  h->launches++;
  SWM_CK(cudaGetLastError());
  SWM_CK(cudaStreamSynchronize(h->stream));
  *out = h;
  return SWM_GPU_OK;
}

int swm_helm_destroy(swm_helm *h) {
  SWM_ON_DEVICE(h ? h->device : -1);
  helm_free(h);
  return SWM_GPU_OK;
}

void *swm_helm_stream(swm_helm *h) { return h ? (void *)h->stream : nullptr; }
int64_t swm_helm_launch_count(swm_helm *h) { return h ? h->launches : -1; }

// out = A psi (ocean cells; 0 elsewhere), FP64
int swm_helm_apply(swm_helm *h, const double *psi, double *out) {
  SWM_ON_DEVICE(h ? h->device : -1);
  SWM_REQUIRE(h && psi && out, "swm_helm_apply: bad arguments");
  SWM_CK(cudaMemcpyAsync(h->psi, psi, h->n * 8, cudaMemcpyHostToDevice, h->stream));
  SWM_CK(cudaMemsetAsync(h->rhs, 0, h->n * 8, h->stream));
  double r2;
  HTRY(resid2<double>(h, h->hinv, h->rhs, h->psi, h->r, &r2));  // r = 0 - A psi
  std::vector<double> t(h->n);
  SWM_CK(cudaMemcpy(t.data(), h->r, h->n * 8, cudaMemcpyDeviceToHost));
  for (size_t k = 0; k < h->n; k++) out[k] = -t[k];
  return SWM_GPU_OK;
}

// FP64 red-black SOR from psi (in/out) to ||rhs - A psi|| < rtol ||rhs||
// (checked every 16 sweeps) or max_sweeps.
int swm_helm_solve_fp64(swm_helm *h, const double *rhs, double *psi, double omega, double rtol, int max_sweeps,
                        int *sweeps, double *relres) {
  SWM_ON_DEVICE(h ? h->device : -1);
  SWM_REQUIRE(h && rhs && psi && max_sweeps > 0, "swm_helm_solve_fp64: bad arguments");
  SWM_CK(cudaMemcpyAsync(h->rhs, rhs, h->n * 8, cudaMemcpyHostToDevice, h->stream));
  SWM_CK(cudaMemcpyAsync(h->psi, psi, h->n * 8, cudaMemcpyHostToDevice, h->stream));
  double bn;
  HTRY(rhs_norm(h, &bn));
  HTRY(split64_setup(h));
  split64_field(h, h->rhs, h->s64.rhs, 0);
  split64_field(h, h->psi, h->s64.psi, 0);
  int s = 0;
  double rel = 1.;
  while (s < max_sweeps) {
    int blk = std::min(HELM_CHECK, max_sweeps - s);
    for (int q = 0; q < blk; q++) sweep64(h, omega);
    s += blk;
    split64_field(h, h->psi, h->s64.psi, 1);  // the residual reads the natural layout
    double r2;
    HTRY(resid2<double>(h, h->hinv, h->rhs, h->psi, nullptr, &r2));
    rel = bn > 0 ? std::sqrt(r2) / bn : std::sqrt(r2);
    if (rel < rtol) break;
  }
  SWM_CK(cudaMemcpyAsync(psi, h->psi, h->n * 8, cudaMemcpyDeviceToHost, h->stream));
  SWM_CK(cudaStreamSynchronize(h->stream));
  if (sweeps) *sweeps = s;
  if (relres) *relres = rel;
  if (rel < rtol) return SWM_GPU_OK;
  set_error("swm_helm_solve_fp64: relative residual above rtol after max_sweeps");
  return SWM_GPU_ENOT_CONVERGED;
}

// Mixed precision: residual r = rhs - A psi in FP64, FP32 SOR sweeps on
// A e = r / ||r|| until its residual falls by inner_tol, psi += ||r|| e in
// FP64; repeated until the FP64 relative residual is below rtol.
int swm_helm_solve_mixed(swm_helm *h, const double *rhs, double *psi, double omega, double rtol, double inner_tol,
                         int max_sweeps, int *sweeps, int *outer, double *relres) {
  SWM_ON_DEVICE(h ? h->device : -1);
  SWM_REQUIRE(h && rhs && psi && max_sweeps > 0 && inner_tol > 0, "swm_helm_solve_mixed: bad arguments");
  SWM_CK(cudaMemcpyAsync(h->rhs, rhs, h->n * 8, cudaMemcpyHostToDevice, h->stream));
  SWM_CK(cudaMemcpyAsync(h->psi, psi, h->n * 8, cudaMemcpyHostToDevice, h->stream));
  double bn;
  HTRY(rhs_norm(h, &bn));
  const unsigned nb = (unsigned)((h->n + 255) / 256);
  int s = 0, o = 0;
  double rel = 1.;
  for (;;) {
    double r2;
    HTRY(resid2<double>(h, h->hinv, h->rhs, h->psi, h->r, &r2));
    const double rn = std::sqrt(r2);
    rel = bn > 0 ? rn / bn : rn;
    if (rel < rtol || s >= max_sweeps || rn == 0.) break;
    k_h_to32<<<nb, 256, 0, h->stream>>>(h->r, h->r32, h->e32, h->n, 1. / rn);
    int si = 0;
    double ri;
    HTRY(inner32(h, (float)omega, inner_tol, max_sweeps - s, &si, &ri));
    k_h_axpy<<<nb, 256, 0, h->stream>>>(h->psi, h->e32, h->n, rn);
    h->launches += 2;
    s += si;
    o++;
  }
  SWM_CK(cudaGetLastError());
  SWM_CK(cudaMemcpyAsync(psi, h->psi, h->n * 8, cudaMemcpyDeviceToHost, h->stream));
  SWM_CK(cudaStreamSynchronize(h->stream));
  if (sweeps) *sweeps = s;
  if (outer) *outer = o;
  if (relres) *relres = rel;
  if (rel < rtol) return SWM_GPU_OK;
  set_error("swm_helm_solve_mixed: relative residual above rtol after max_sweeps");
  return SWM_GPU_ENOT_CONVERGED;
}

// Autotuner: the sweep kernel's block shape by timing FP32 sweeps, then the
// relaxation factor in [omega_lo, omega_hi] (ngrid values) as the one whose
// trial solve of trial_sweeps FP32 sweeps on A e = rhs / ||rhs|| from e = 0
// reaches the smallest residual.
int swm_helm_autotune(swm_helm *h, const double *rhs, double omega_lo, double omega_hi, int ngrid,
                      int trial_sweeps, double *omega, int *block_x, int *block_y) {
  SWM_ON_DEVICE(h ? h->device : -1);
  SWM_REQUIRE(h && rhs && ngrid >= 1 && trial_sweeps > 0 && omega_lo > 0 && omega_hi < 2 && omega_lo <= omega_hi,
              "swm_helm_autotune: bad arguments");
  SWM_CK(cudaMemcpyAsync(h->rhs, rhs, h->n * 8, cudaMemcpyHostToDevice, h->stream));
  double bn;
  HTRY(rhs_norm(h, &bn));
  const unsigned nb = (unsigned)((h->n + 255) / 256);
  k_h_to32<<<nb, 256, 0, h->stream>>>(h->rhs, h->r32, h->e32, h->n, bn > 0 ? 1. / bn : 1.);
  h->launches++;
  // block shape
  const dim3 shapes[4] = {dim3(32, 8), dim3(64, 4), dim3(128, 2), dim3(256, 1)};
  cudaEvent_t a, b;
  int best_k = 4;
  SWM_CK(cudaEventCreate(&a));
  SWM_CK(cudaEventCreate(&b));
  float tbest = 1e30f;
  for (const dim3 &shp : shapes) {
    sweep32(h, 1.f, shp);
    SWM_CK(cudaEventRecord(a, h->stream));
    for (int q = 0; q < 4; q++) sweep32(h, 1.f, shp);
    SWM_CK(cudaEventRecord(b, h->stream));
    SWM_CK(cudaEventSynchronize(b));
    float ms;
    SWM_CK(cudaEventElapsedTime(&ms, a, b));
    if (ms < tbest) { tbest = ms; h->blk = shp; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  // sweeps per temporally blocked launch (SWM_GB300_HELM_K overrides; 0:
  // global sweeps only)
  const char *ek = getenv("SWM_GB300_HELM_K");
  if (ek && atoi(ek) >= 0 && atoi(ek) <= 4 && ek[0] >= '0' && ek[0] <= '9') {
    h->tbk = atoi(ek);
  } else {
    SWM_CK(cudaEventCreate(&a));
    SWM_CK(cudaEventCreate(&b));
    float kbest = 1e30f;
    for (int kk : {1, 2, 3, 4}) {
      h->tbk = kk;
      sweeps_tb32(h, 1.f, 4);
      SWM_CK(cudaEventRecord(a, h->stream));
      sweeps_tb32(h, 1.f, 8);
      SWM_CK(cudaEventRecord(b, h->stream));
      SWM_CK(cudaEventSynchronize(b));
      float ms;
      SWM_CK(cudaEventElapsedTime(&ms, a, b));
      if (ms < kbest) { kbest = ms; best_k = kk; }
    }
    h->tbk = best_k;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  // relaxation factor
  double best = omega_lo, rbest = 1e300;
  for (int q = 0; q < ngrid; q++) {
    const double om = ngrid == 1 ? omega_lo : omega_lo + (omega_hi - omega_lo) * q / (ngrid - 1);
    k_h_to32<<<nb, 256, 0, h->stream>>>(h->rhs, h->r32, h->e32, h->n, bn > 0 ? 1. / bn : 1.);
    h->launches++;
    const int tb = tb_part(h, trial_sweeps);
    sweeps_tb32(h, (float)om, tb);
    for (int s = tb; s < trial_sweeps; s++) sweep32(h, (float)om, h->blk);
    double e2;
    HTRY(resid2<float>(h, h->hinv32, h->r32, h->e32, nullptr, &e2));
    if (e2 < rbest) { rbest = e2; best = om; }
  }
  if (omega) *omega = best;
  if (block_x) *block_x = (int)h->blk.x;
  if (block_y) *block_y = (int)h->blk.y;
  return SWM_GPU_OK;
}

}  // extern "C"
