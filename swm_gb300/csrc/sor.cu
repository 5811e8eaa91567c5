// sor.cu -- red-black SOR of ElSolv_SOR.f90 on the GPU.
//
// Reference semantics: 5-point masked spherical Laplacian coefficients
// (init_ElSolv_SOR :54-62), colour 1 = i+j even (1-based) then colour 2,
// fixed Chebyshev relaxation schedule from rJacobi = 0.99999178 (binary32
// literal, :175, :206-210), stop on the first iteration whose correction norm
// sqrt(sum res^2) drops below eps (:213-218), max_count = 1000 max(Nx, Ny)
// on a first call and 10 max(Nx, Ny) after it (:166-176).
//
// Layout: the coefficients, the right-hand side, chi and the ocean mask are
// kept split by colour, row by row: cell (i, j) of colour (i + j) % 2 sits at
// j * W + i / 2 of its colour's arrays (W = ceil(Nx / 2)).  A half-sweep then
// reads only its own colour's coefficients, right-hand side, reciprocal
// diagonal and chi (and the other colour's chi as neighbours): 10 words per
// point and iteration, SOR_CELLS consecutive cells of the colour per thread,
// coalesced.  Each cell's update is the reference's expression in the
// reference's order (this file is compiled without FMA contraction), so chi
// is bit for bit the restatement's when the iteration counts agree; within a
// colour no cell reads another of its own colour (the periodic wrap only
// pairs land cells, which stay fixed).
//
// Division: GB300's FP64 rate is low and the half-sweep is bound by it, so
// the update's division by the diagonal coefficient is formed from that
// coefficient's reciprocal, set up once, by Markstein's correction
// (div_rn below): the same correctly rounded quotient with five FP64
// operations.
//
// Control: the relaxation factor, the iteration counter and the stop flag
// live on the device.  Each half-sweep kernel sums res^2 per warp with
// shuffles and per block; the last block to finish (fence and counter) adds
// the blocks in a fixed order, advances the relaxation schedule, and after
// the second colour applies the stop test.  The kernels take no per-
// iteration arguments, so a batch of iterations is one CUDA graph, replayed
// until the flag is set; kernels after convergence (or max_count) return at
// once.  The host reads the flag once per batch.
#include <cmath>
#include <string>
#include <vector>
#include "ctx.h"
#include "divide.cuh"

// device control block of a solve
struct SorCtl {
  double relax;      // relaxation factor of the next half-sweep
  double sum0;       // sum of res^2 of the current iteration's first colour
  double anorm;      // correction norm of the last finished iteration
  double eps;        // stop when the correction norm falls below it
  int l;             // the iteration the next half-sweep belongs to (1-based)
  int max_count;
  int done;          // 1: converged (at iteration iters)
  int iters;
  unsigned count;    // blocks finished in the running half-sweep
};

struct SorState {
  double *c[5] = {};       // ElSolvSOR_c(:,:,1..5), natural layout (set-up only)
  double *chi = nullptr, *B = nullptr;   // natural layout; chi: calc_lib::chi, kept between
                                         // swm_gpu_nondivergent calls
  double *chi_io = nullptr;              // natural layout: elsolv_sor_gpu_solve's chi
  double *cs[2][5] = {};   // coefficients split by colour
  double *rc4[2] = {};     // 1 / ElSolvSOR_c(:,:,5), split by colour
  uint8_t *ms[2] = {};     // ocean mask split by colour (0 also on the padding of odd rows)
  int *bad = nullptr;      // set-up: 1 when an ocean cell's diagonal is outside div_rn's range
  bool fast = true;        // every ocean diagonal inside div_rn's range
  double *Bs[2] = {}, *chis[2] = {};     // right-hand side and chi split by colour
  double *partial = nullptr;   // per-block sums of res^2 of a half-sweep
  SorCtl *ctl = nullptr;
  double *und = nullptr, *vnd = nullptr;  // non-divergent flow
  int W = 0, nblocks = 0;      // split row length; blocks of a half-sweep
  cudaGraphExec_t graph = nullptr;  // SOR_BATCH iterations
};

constexpr int SOR_THREADS = 256;
constexpr int SOR_CELLS = 4;  // consecutive cells of the colour per thread (one 32-bit word of mask bytes)
constexpr int SOR_BATCH = 32;  // iterations per graph replay (one host read of the flag)

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

// natural <-> colour-split layout (join 0: natural -> split, 1: split -> natural)
__global__ void k_sor_split(double *nat, double *s0, double *s1, int nx, int ny, int W, int join) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)nx * ny) return;
  const int i = (int)(k % nx), j = (int)(k / nx);
  double *sp = ((i + j) & 1) ? s1 : s0;
  const size_t q = (size_t)j * W + (i >> 1);
  if (join) nat[k] = sp[q];
  else sp[q] = nat[k];
}

// set-up: the reciprocal diagonal and the split ocean mask of colour col;
// *bad = 1 when an ocean cell's diagonal is outside div_rn's range
__global__ void k_sor_recip(const int8_t *__restrict__ ocean, const double *__restrict__ c4, double *__restrict__ rc4,
                            uint8_t *__restrict__ ms, int nx, int ny, int W, int col, int *bad) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)W * ny) return;
  const int j = (int)(q / W), i = 2 * (int)(q % W) + ((col + j) & 1);
  const bool o = i < nx && ocean[i + (size_t)nx * j] != 0;
  ms[q] = o;
  rc4[q] = 1. / c4[q];
  if (o && !div_rn_range(c4[q])) atomicOr(bad, 1);
}

// One half-sweep of colour col (0: (i+j) even in 0-based indices, the
// reference's colour 1) over the colour-split arrays, SOR_CELLS cells per
// thread; then the block sums of res^2 and, in the last block, the
// iteration's bookkeeping.  FAST: the division by div_rn (every ocean
// diagonal in its range; a numerator outside it still divides).
template <bool FAST>
__global__ void __launch_bounds__(SOR_THREADS) k_sor_half(SorState s, int nx, int ny, int col, double rJ) {
  SorCtl *ctl = s.ctl;
  if (ctl->done || ctl->l > ctl->max_count) return;  // converged, or max_count reached
  const double relax = ctl->relax;
  const int W = s.W;
  const size_t ns = (size_t)W * ny;
  const size_t q0 = ((size_t)blockIdx.x * SOR_THREADS + threadIdx.x) * SOR_CELLS;
  const double *const *cs = s.cs[col];
  double *x = s.chis[col];
  double r2 = 0.;
  if (q0 < ns) {
    uint32_t m4 = 0;  // the cells' mask bytes
    if (q0 + SOR_CELLS <= ns) {
      m4 = *reinterpret_cast<const uint32_t *>(s.ms[col] + q0);
    } else {
      for (int k = 0; k < SOR_CELLS && q0 + k < ns; k++) m4 |= (uint32_t)s.ms[col][q0 + k] << (8 * k);
    }
#pragma unroll
    for (int k = 0; k < SOR_CELLS; k++) {
      if (!((m4 >> (8 * k)) & 0xffu)) continue;
      const size_t q = q0 + k;
      const int j = (int)(q / W), i = 2 * (int)(q - (size_t)j * W) + ((col + j) & 1);
      const int ip = i + 1 == nx ? 0 : i + 1, im = i == 0 ? nx - 1 : i - 1;
      const int jp = j + 1 == ny ? 0 : j + 1, jm = j == 0 ? ny - 1 : j - 1;
      // neighbours are of the other colour except across an odd periodic wrap
      auto at = [&](int a, int b) { return s.chis[(a + b) & 1][(size_t)b * W + (a >> 1)]; };
      const double c4 = cs[4][q];
      const double num = relax * (cs[0][q] * at(ip, j) + cs[1][q] * at(im, j) + cs[2][q] * at(i, jp) +
                                  cs[3][q] * at(i, jm) + c4 * x[q] - s.Bs[col][q]);
      const double res = FAST && div_rn_range(num) ? div_rn(num, c4, s.rc4[col][q]) : num / c4;
      x[q] = x[q] - res;
      r2 = r2 + res * res;
    }
  }
  // block sum: shuffles within warps, then the warps in order
  __shared__ double wsum[SOR_THREADS / 32];
  __shared__ bool last;
  for (int o = 16; o > 0; o >>= 1) r2 += __shfl_down_sync(0xffffffffu, r2, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = r2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.;
    for (int w = 0; w < SOR_THREADS / 32; w++) b += wsum[w];
    s.partial[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(&ctl->count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  // last block: the blocks' sums in block order (thread t adds blocks t,
  // t + 256, ..., then the warps' shuffle trees, then the warps in order)
  __threadfence();
  double v = 0.;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += SOR_THREADS) v += ((volatile double *)s.partial)[b];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < SOR_THREADS / 32; w++) tot += wsum[w];
    const int l = ctl->l;
    // the schedule of main_ElSolv_SOR (:206-210): after the first colour of
    // the first iteration 1 / (1 - rJ^2 / 2), else 1 / (1 - rJ^2 relax / 4)
    if (col == 0 && l == 1) ctl->relax = 1. / (1. - .5 * rJ * rJ);
    else ctl->relax = 1. / (1. - .25 * rJ * rJ * relax);
    if (col == 0) {
      ctl->sum0 = tot;
    } else {
      const double an = sqrt(ctl->sum0 + tot);
      ctl->anorm = an;
      if (an < ctl->eps) {
        ctl->done = 1;
        ctl->iters = l;
      }
      ctl->l = l + 1;
    }
    ctl->count = 0;
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

// the pair of k_div_check's sample k: splitmix64 bits; one pair in four
// takes a special significand (all ones, all zeros, or one of them with the
// lowest bits flipped) for a, b or both; one numerator in eight lies
// outside div_rn's range (zeros, subnormal, tiny, huge, infinite, NaN), so
// div_fast's other branches are checked too
__device__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ double sample_operand(uint64_t r, uint64_t r2, bool special) {
  uint64_t man = r & 0xfffffffffffffull;
  if (special) {
    const uint64_t pat[4] = {0xfffffffffffffull, 0ull, 0xffffffffffff0ull ^ (r2 & 15), r2 & 15};
    man = pat[(r2 >> 8) & 3];
  }
  const uint64_t e = 523 + (r2 >> 16) % 1001;  // binary exponent -500 .. 500
  const uint64_t sign = (r2 >> 40) & 1;
  return __longlong_as_double((long long)((sign << 63) | (e << 52) | man));
}

__global__ void k_div_check(int64_t n, uint64_t seed, unsigned long long *bad) {
  unsigned long long mism = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h = mix64(seed ^ mix64((uint64_t)k));
    const uint64_t r[4] = {mix64(h + 1), mix64(h + 2), mix64(h + 3), mix64(h + 4)};
    const int sp = (int)(h & 15);  // 0, 1, 2: special a, b, both
    double a = sample_operand(r[0], r[1], sp == 0 || sp == 2);
    const double b = sample_operand(r[2], r[3], sp == 1 || sp == 2);
    if (((h >> 4) & 7) == 0) {  // one sample in eight: a numerator outside div_rn's range
      const uint64_t sign = (r[1] >> 41) & 1, man = r[0] & 0xfffffffffffffull;
      const uint64_t lo = 1 + (r[1] >> 16) % 522, hi = 1524 + (r[1] >> 16) % 523;  // exponent fields
      const uint64_t bits[8] = {0, 0, man, lo << 52 | man, hi << 52 | man, 0x7ffull << 52, 0x7ffull << 52,
                                0x7ffull << 52 | 1};  // +-0, subnormal, tiny, huge, inf, inf, NaN
      a = __longlong_as_double((long long)((sign << 63) | bits[(h >> 7) & 7]));
    }
    const double q = __ddiv_rn(a, b), y = __ddiv_rn(1., b), f = div_fast(a, b, y);
    const bool same = __double_as_longlong(f) == __double_as_longlong(q) || (q != q && f != f);
    mism += !same;
  }
  for (int o = 16; o > 0; o >>= 1) mism += __shfl_down_sync(0xffffffffu, mism, o);
  if ((threadIdx.x & 31) == 0 && mism) atomicAdd(bad, mism);
}

void sor_free(swm_gpu_ctx *c) {
  if (!c->sor) return;
  SorState *s = c->sor;
  if (s->graph) cudaGraphExecDestroy(s->graph);
  for (int q = 0; q < 5; q++) cudaFree(s->c[q]);
  for (int col = 0; col < 2; col++) {
    for (int q = 0; q < 5; q++) cudaFree(s->cs[col][q]);
    cudaFree(s->Bs[col]);
    cudaFree(s->chis[col]);
    cudaFree(s->rc4[col]);
    cudaFree(s->ms[col]);
  }
  cudaFree(s->bad);
  cudaFree(s->chi); cudaFree(s->chi_io); cudaFree(s->B); cudaFree(s->partial); cudaFree(s->ctl);
  cudaFree(s->und); cudaFree(s->vnd);
  delete s;
  c->sor = nullptr;
}

}  // namespace swm

using namespace swm;

extern "C" {

int elsolv_sor_gpu_init(swm_gpu_ctx *c) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 1, "elsolv_sor_gpu_init: call after swm_gpu_domain");
  sor_free(c);
  SorState *s = new SorState();
  c->sor = s;
  const size_t n = c->n;
  s->W = (c->nx + 1) / 2;
  const size_t ns = (size_t)s->W * c->ny;
  s->nblocks = (int)((ns + (size_t)SOR_THREADS * SOR_CELLS - 1) / ((size_t)SOR_THREADS * SOR_CELLS));
  for (int q = 0; q < 5; q++) SWM_CK(cudaMalloc((void **)&s->c[q], n * 8));
  for (int col = 0; col < 2; col++) {
    for (int q = 0; q < 5; q++) SWM_CK(cudaMalloc((void **)&s->cs[col][q], ns * 8));
    SWM_CK(cudaMalloc((void **)&s->Bs[col], ns * 8));
    SWM_CK(cudaMalloc((void **)&s->chis[col], ns * 8));
    SWM_CK(cudaMalloc((void **)&s->rc4[col], ns * 8));
    SWM_CK(cudaMalloc((void **)&s->ms[col], ns + SOR_CELLS));
  }
  SWM_CK(cudaMalloc((void **)&s->bad, sizeof(int)));
  SWM_CK(cudaMemsetAsync(s->bad, 0, sizeof(int), c->stream));
  SWM_CK(cudaMalloc((void **)&s->chi, n * 8));
  SWM_CK(cudaMalloc((void **)&s->chi_io, n * 8));
  SWM_CK(cudaMalloc((void **)&s->B, n * 8));
  SWM_CK(cudaMalloc((void **)&s->partial, (size_t)s->nblocks * 8));
  SWM_CK(cudaMalloc((void **)&s->ctl, sizeof(SorCtl)));
  SWM_CK(cudaMemsetAsync(s->ctl, 0, sizeof(SorCtl), c->stream));
  SWM_CK(cudaMemsetAsync(s->chi, 0, n * 8, c->stream));  // calc_lib::chi starts at 0
  dim3 b(32, 8), g((c->nx + 31) / 32, (c->ny + 7) / 8);
  k_sor_coeff<<<g, b, 0, c->stream>>>(c->dev(), *s);
  const unsigned nb = (unsigned)((n + 255) / 256);
  for (int q = 0; q < 5; q++)
    k_sor_split<<<nb, 256, 0, c->stream>>>(s->c[q], s->cs[0][q], s->cs[1][q], c->nx, c->ny, s->W, 0);
  const unsigned nbs = (unsigned)((ns + 255) / 256);
  for (int col = 0; col < 2; col++)
    k_sor_recip<<<nbs, 256, 0, c->stream>>>(c->d_ocean[GE], s->cs[col][4], s->rc4[col], s->ms[col], c->nx, c->ny,
                                            s->W, col, s->bad);
  c->launches += 8;
  SWM_CK(cudaGetLastError());
  int bad = 0;
  SWM_CK(cudaMemcpyAsync(&bad, s->bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  s->fast = bad == 0;
  return SWM_GPU_OK;
}

}  // extern "C"

namespace {

// the two half-sweeps of one iteration
void sor_iteration(swm_gpu_ctx *c, SorState *s) {
  const double rJ = (double)(float)9.9999178e-1;  // default-real literal (ElSolv_SOR.f90:175)
  for (int col = 0; col < 2; col++) {
    if (s->fast) k_sor_half<true><<<s->nblocks, SOR_THREADS, 0, c->stream>>>(*s, c->nx, c->ny, col, rJ);
    else k_sor_half<false><<<s->nblocks, SOR_THREADS, 0, c->stream>>>(*s, c->nx, c->ny, col, rJ);
  }
}

// SOR_BATCH iterations as one graph, captured once per set-up (the kernels
// read their iteration state and eps from the control block, so one capture
// serves every batch and every call)
int sor_graph(swm_gpu_ctx *c, SorState *s) {
  if (s->graph) return SWM_GPU_OK;
  SWM_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int l = 0; l < SOR_BATCH; l++) sor_iteration(c, s);
  cudaGraph_t g = nullptr;
  SWM_CK(cudaStreamEndCapture(c->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    s->graph = nullptr;
    set_error(std::string("elsolv_sor_gpu_solve: cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return SWM_GPU_ECUDA;
  }
  return SWM_GPU_OK;
}

}  // namespace

// main_ElSolv_SOR on the device arrays s->B (right-hand side) and chi
// (first guess in, solution out), natural layout; returns
// SWM_GPU_ENOT_CONVERGED after max_count iterations
static int sor_solve_device(swm_gpu_ctx *c, double *chi, double eps, int first_guess, int *iters, double *anorm) {
  SorState *s = c->sor;
  const int mx = c->nx > c->ny ? c->nx : c->ny;
  const int max_count = first_guess ? (int)lround(1000. * mx) : (int)lround(10. * mx);
  const unsigned nb = (unsigned)((c->n + 255) / 256);
  k_sor_split<<<nb, 256, 0, c->stream>>>(s->B, s->Bs[0], s->Bs[1], c->nx, c->ny, s->W, 0);
  k_sor_split<<<nb, 256, 0, c->stream>>>(chi, s->chis[0], s->chis[1], c->nx, c->ny, s->W, 0);
  c->launches += 2;
  SorCtl ctl = {};
  ctl.relax = 1.;
  ctl.l = 1;
  ctl.max_count = max_count;
  ctl.eps = eps;
  SWM_CK(cudaMemcpyAsync(s->ctl, &ctl, sizeof(SorCtl), cudaMemcpyHostToDevice, c->stream));
  int rc = sor_graph(c, s);
  if (rc != SWM_GPU_OK) return rc;
  for (int l = 1; l <= max_count; l += SOR_BATCH) {
    SWM_CK(cudaGraphLaunch(s->graph, c->stream));
    c->launches += 2 * SOR_BATCH;
    SWM_CK(cudaMemcpyAsync(&ctl, s->ctl, sizeof(SorCtl), cudaMemcpyDeviceToHost, c->stream));
    SWM_CK(cudaStreamSynchronize(c->stream));
    if (ctl.done) break;
  }
  k_sor_split<<<nb, 256, 0, c->stream>>>(chi, s->chis[0], s->chis[1], c->nx, c->ny, s->W, 1);
  c->launches++;
  SWM_CK(cudaGetLastError());
  if (anorm) *anorm = ctl.anorm;
  if (ctl.done) {
    if (iters) *iters = ctl.iters;
    return SWM_GPU_OK;
  }
  if (iters) *iters = max_count;
  set_error("elsolv_sor_gpu_solve: not converged after max_count iterations");
  return SWM_GPU_ENOT_CONVERGED;
}

extern "C" {

int elsolv_sor_gpu_solve(swm_gpu_ctx *c, const double *B, double *chi, double eps, int first_guess, int *iters,
                         double *anorm) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->sor && B && chi, "elsolv_sor_gpu_solve: call elsolv_sor_gpu_init first");
  SorState *s = c->sor;
  size_t n = c->n;
  SWM_CK(cudaMemcpyAsync(s->B, B, n * 8, cudaMemcpyHostToDevice, c->stream));
  SWM_CK(cudaMemcpyAsync(s->chi_io, chi, n * 8, cudaMemcpyHostToDevice, c->stream));
  int rc = sor_solve_device(c, s->chi_io, eps, first_guess, iters, anorm);
  SWM_CK(cudaMemcpyAsync(chi, s->chi_io, n * 8, cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return rc;
}

int swm_gpu_check_division(int64_t n, int64_t seed, int64_t *mismatches) {
  SWM_REQUIRE(n >= 0 && mismatches, "swm_gpu_check_division: bad arguments");
  unsigned long long *d = nullptr;
  SWM_CK(cudaMalloc((void **)&d, sizeof(*d)));
  cudaError_t e = cudaMemset(d, 0, sizeof(*d));
  if (e == cudaSuccess) {
    k_div_check<<<4 * 152, 256>>>(n, (uint64_t)seed, d);
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error(std::string("swm_gpu_check_division: ") + cudaGetErrorString(e));
    return SWM_GPU_ECUDA;
  }
  *mismatches = (int64_t)h;
  return SWM_GPU_OK;
}

// computeNonDivergentFlowField (calc_lib.f90:548-590) of the model's current
// (u, v): divergence, SOR for chi (chi kept on the device between calls as
// the reference keeps calc_lib::chi; first_guess as itt == 1), gradient,
// u_nd = u - grad_lambda chi, v_nd = v - grad_theta chi.  Outputs may be
// NULL.  SOR non-convergence is reported as by elsolv_sor_gpu_solve, with
// the non-divergent flow still formed.
int swm_gpu_nondivergent(swm_gpu_ctx *c, int first_guess, double eps, double *u_nd, double *v_nd, double *chi,
                         int *iters) {
  SWM_ON_DEVICE(c ? c->device : -1);
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
  int rc = sor_solve_device(c, s->chi, eps, first_guess, iters, nullptr);
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
