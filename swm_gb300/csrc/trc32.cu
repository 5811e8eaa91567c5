// trc32.cu -- passive tracers on the FP32 compensated path, all tracers of a
// basin in one kernel per step.
//
// Formulas: TRC_tracer_incr (tracer_module.f90:154-209), TRC_initCoeffs
// (:291-342, coefficients rebuilt from the masks and per-row metric factors,
// with the 0/0 of land-land pairs taken as 0), TRC_tracer_integrate
// (:216-232); thickness and face thicknesses as computeD
// (swm_nonlinear_timestep_module.f90:182-218).  The tracer content CH is a
// (hi, lo) binary32 pair with a compensated Adams-Bashforth update and the
// implicit decay applied as x - x*dt*cons/(1 + dt*cons); increments are
// binary32.  Extension: third-order upwind-biased face values
// (swm_gpu_config.tracer_flux = 1) with the reference's mask-weighted mean
// next to land.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "ctx.h"
#include "fused32.h"

namespace swm {

constexpr int TRC32_MAX = 4;  // tracers per launch (more run in several launches)
enum { RT_RDL, RT_RDT, RT_CV, RT_D8, RT_D10, RT_NR };

struct Tracer32 {
  float *ch[2] = {}, *cl[2] = {};  // CH pair, levels TRC_N0 / TRC_N0p1 (rotated)
  float *G[3] = {};
  float *C0 = nullptr, *gamma = nullptr, *dp = nullptr;  // fields, or null when uniform
  float gamma_s = 0.f, dp_s = 0.f, kappa = 0.f;
  int n0 = 0, g0 = 0;
};

struct TrcP {
  int nx, ny, nl, flux, ntr, pf;
  float dt, ab0, ab1, ab2;
  const float *u, *v, *eta, *He, *Fe, *rows;
  const uint16_t *mask16;
  struct {
    const float *ch, *cl, *G1, *G2, *C0, *gamma, *dp;
    float *chn, *cln, *G3;
    float gamma_s, dp_s, kappa;
  } t[TRC32_MAX];
};

__device__ __forceinline__ int wr(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// 1 / thickness, 0 on dry land (C = CH * rD then takes the 0/0 there as 0)
__device__ __forceinline__ float rthick(float d) { return d != 0.f ? __frcp_rn(d) : 0.f; }

// face value of CH between L and R (R east/north of L), Lm behind L, Rp beyond R
__device__ __forceinline__ float face(int flux, float vel, float cLm, float cL, float cR, float cRp, unsigned oLm,
                                      unsigned oL, unsigned oR, unsigned oRp) {
  if (flux == 1 && oLm && oL && oR && oRp)
    return vel >= 0.f ? (5.f * cL + 2.f * cR - cLm) * (1.f / 6.f) : (2.f * cL + 5.f * cR - cRp) * (1.f / 6.f);
  unsigned den = oL + oR;
  if (den == 0) return 0.f;
  return (oL ? cL : 0.f) * (den == 2 ? 0.5f : 1.f) + (oR ? cR : 0.f) * (den == 2 ? 0.5f : 1.f);
}

// (hi + lo + inc) * (1 - dp) as a new (hi, lo) pair, the two roundings
// recovered by Fast2Sum (Dekker 1971): exact for s - c (c = s dp, 0 <= dp <
// 1), and for hi + inc wherever the increment is below the tracer content,
// which fails only where the content passes through zero
__device__ __forceinline__ void comp_update(float hi, float lo, float inc, float dp, float &nh, float &nl) {
  const float s = hi + inc;
  float e = (inc - (s - hi)) + lo;
  const float c = s * dp;
  const float t = s - c;
  const float e2 = (s - t) - c;
  e = e + e2 - e * dp;
  nh = t + e;
  nl = e - (nh - t);
}

constexpr unsigned FULLM = 0xffffffffu;
constexpr int TRC_ROWS = 16;  // output rows per warp

// One warp owns a strip of 32 columns (lane = column; 2 halo lanes per side,
// as the upwind-biased faces reach two cells) and TRC_ROWS output rows; it
// walks up the strip keeping the last five rows of CH (hi + lo), thickness
// and masks in registers, and updates row J-2 once row J is in.
// PF 1: each iteration also asks L2 for the input rows two beyond those it
// loads and for the update inputs of the output row after next, so that a
// state larger than L2 does not make the warp wait on DRAM (trc_prefetch).
// Resident blocks per SM asked of the register allocator: one tracer fits 6
// (80 registers, no spill; 2049^2 step 76.0 us against 83.8 at 4), two
// tracers 4 (at 5 they spill and run slower), three 4 with the updated row's
// CH pair reloaded instead of carried (RELOAD; 2049^2 step 169 us against
// 176 at 3 blocks), four 3.
template <int NT, int FLUX, int PF>
__global__ void __launch_bounds__(128, NT == 1 ? 6 : (NT <= 3 ? 4 : 3)) k_trc32(TrcP p, int S, int nstrips) {
  constexpr bool RELOAD = NT == 3;
  constexpr int H = 2, TI = 32 - 2 * H;
  const int lane = threadIdx.x & 31;
  // block b: strip b % nstrips, its four warps four consecutive row groups
  const int nx = p.nx, ny = p.ny;
  const int ry0 = ((blockIdx.x / nstrips) * 4 + (threadIdx.x >> 5)) * S;
  if (ry0 >= ny) return;  // whole warp leaves together
  const int gx = (blockIdx.x % nstrips) * TI - H + lane;
  const int gi = wr(gx, nx);
  const bool store_lane = lane >= H && lane < 32 - H && gx < nx;

  unsigned m[5] = {};
  float D[5] = {}, rD[5] = {}, u[3] = {}, v[3] = {};
  float chs[NT][5] = {}, chh[NT][3] = {}, chl[NT][3] = {};
  int off[3] = {};
  const float *rr[3] = {};

  int J = ry0 - 2;
  const int ylast = min(ry0 + S, ny);  // one past the last output row
  const int jend = ylast + 2;
  // row loads run two rows ahead of the window; the update inputs (increments
  // 1-2, C0) one output row ahead
  struct Row {
    unsigned m;
    float D, u, v, h[NT], l[NT];
    int off;
    const float *rows;
  };
  auto load = [&](int jj, Row &r) {
    const int jw = wr(jj, ny);
    r.off = nx * jw;
    r.rows = p.rows + (size_t)jw * RT_NR;
    const int k = gi + r.off;
    r.m = p.mask16[k];
    r.D = p.nl ? ((r.m & 8u) ? p.He[k] + p.eta[k] : 1.f) : p.He[k];
    r.u = p.u[k];
    r.v = p.v[k];
#pragma unroll
    for (int q = 0; q < NT; q++) {
      r.h[q] = p.t[q].ch[k];
      r.l[q] = p.t[q].cl[k];
    }
  };
  Row n1, n2;
  load(J, n1);
  load(J + 1, n2);
  float pg1[NT] = {}, pg2[NT] = {}, pc0[NT] = {};
  float fyp[NT] = {};  // flux through the north faces of the previous output row

  for (; J < jend; J++) {
#pragma unroll
    for (int a = 4; a > 0; a--) {
      m[a] = m[a - 1];
      D[a] = D[a - 1];
      rD[a] = rD[a - 1];
#pragma unroll
      for (int q = 0; q < NT; q++) chs[q][a] = chs[q][a - 1];
    }
#pragma unroll
    for (int a = 2; a > 0; a--) {
      u[a] = u[a - 1];
      v[a] = v[a - 1];
      off[a] = off[a - 1];
      rr[a] = rr[a - 1];
#pragma unroll
      for (int q = 0; q < NT; q++) {
        if (!RELOAD) {
          chh[q][a] = chh[q][a - 1];
          chl[q][a] = chl[q][a - 1];
        }
      }
    }
    m[0] = n1.m; D[0] = n1.D; rD[0] = rthick(n1.D); u[0] = n1.u; v[0] = n1.v; off[0] = n1.off; rr[0] = n1.rows;
#pragma unroll
    for (int q = 0; q < NT; q++) {
      if (!RELOAD) {
        chh[q][0] = n1.h[q];
        chl[q][0] = n1.l[q];
      }
      chs[q][0] = n1.h[q] + n1.l[q];
    }
    n1 = n2;
    if (J + 2 < jend) load(J + 2, n2);
    if (PF) {
      if (J + 4 < jend) {  // rows two beyond the one just loaded
        const int k4 = gi + nx * wr(J + 4, ny);
        prefetch_l2(p.mask16 + k4);
        prefetch_l2(p.He + k4);
        if (p.nl) prefetch_l2(p.eta + k4);
        prefetch_l2(p.u + k4);
        prefetch_l2(p.v + k4);
#pragma unroll
        for (int q = 0; q < NT; q++) {
          prefetch_l2(p.t[q].ch + k4);
          prefetch_l2(p.t[q].cl + k4);
        }
      }
      if (store_lane && J >= ry0 && J < ylast) {  // update inputs of output row J (loaded at J + 1)
        const int k0 = gi + off[0];
#pragma unroll
        for (int q = 0; q < NT; q++) {
          prefetch_l2(p.t[q].G1 + k0);
          prefetch_l2(p.t[q].G2 + k0);
          prefetch_l2(p.t[q].C0 + k0);
        }
      }
    }

    const int o = J - 2;
    // row ry0 - 1 only forms its north faces (the south faces of row ry0)
    if (o >= ry0 - 1) {  // uniform across the warp
      const bool upd = store_lane && o >= ry0 && o < ny;
      // masks of row o and its neighbours
      const unsigned mo = m[2];
      const unsigned oE = (mo >> 3) & 1, oEim = (mo >> 7) & 1, oEip = (mo >> 11) & 1;
      const unsigned oUip = (mo >> 9) & 1, oV = (mo >> 2) & 1;
      const unsigned oVjp = (m[1] >> 2) & 1, oEjp = (m[1] >> 3) & 1, oEjm = (m[3] >> 3) & 1;
      const unsigned oEipp = (__shfl_down_sync(FULLM, mo, 1) >> 11) & 1;
      const unsigned oEjpp = (m[0] >> 3) & 1;
      const float Do = D[2], Dip = __shfl_down_sync(FULLM, Do, 1);
      const float Djp = D[1], Djm = D[3];
      const float ro = rD[2], rip = __shfl_down_sync(FULLM, ro, 1);
      const float rjp = rD[1], rjm = rD[3];
      const float uip = __shfl_down_sync(FULLM, u[2], 1), vjp = v[1];
      const float *r = rr[2], *rp = rr[1];
      const float cv = r[RT_CV], cvp = rp[RT_CV];
      auto avg2 = [](float a, unsigned oa, float b, unsigned ob) {
        unsigned c = oa + ob;
        return c == 0 ? 0.f : ((oa ? a : 0.f) + (ob ? b : 0.f)) * (c == 2 ? 0.5f : 1.f);
      };
      const float huip = avg2(Dip, oEip, Do, oE);
      const float c8 = oUip * r[RT_D8];
      // Advective fluxes through the east and north faces of every lane's
      // cell, and the diffusive flux through the east face.  The west face
      // of a cell is the east face of the lane below it, the south face the
      // north face of the previous output row: the same operands in the same
      // order, so the same bits as forming them again (and one call site, so
      // one rounding of the contracted arithmetic).
      float fxe[NT], fxw[NT], fyn[NT], fys[NT], dxe[NT], dxw[NT];
#pragma unroll
      for (int q = 0; q < NT; q++) {
        const float ch = chs[q][2], chip = __shfl_down_sync(FULLM, ch, 1), chim = __shfl_up_sync(FULLM, ch, 1);
        const float chrr = FLUX ? __shfl_down_sync(FULLM, ch, 2) : 0.f;
        const float chjp = chs[q][1], chjm = chs[q][3];
        fxe[q] = oUip * uip * face(FLUX, uip, chim, ch, chip, chrr, oEim, oE, oEip, oEipp);
        fyn[q] = oVjp * cvp * vjp * face(FLUX, vjp, chjm, ch, chjp, chs[q][0], oEjm, oE, oEjp, oEjpp);
        fys[q] = fyp[q];
        fyp[q] = fyn[q];
        dxe[q] = huip * (chip * rip - ch * ro) * c8;
        fxw[q] = __shfl_up_sync(FULLM, fxe[q], 1);
        dxw[q] = -__shfl_up_sync(FULLM, dxe[q], 1);
      }
      if (upd) {
        const int ko = gi + off[2];
        const float rdl = r[RT_RDL], rdt = r[RT_RDT];
        const float hv = avg2(Do, oE, Djm, oEjm), hvjp = avg2(Djp, oEjp, Do, oE);
        const float Fe = p.Fe ? p.Fe[ko] : 0.f;
        const float c10 = oVjp * cvp * r[RT_D10], c11 = -(float)oV * cv * r[RT_D10];
#pragma unroll
        for (int q = 0; q < NT; q++) {
          const auto &t = p.t[q];
          const float ch = chs[q][2], chjp = chs[q][1], chjm = chs[q][3];
          float g = rdl * (fxw[q] - fxe[q]) + rdt * (fys[q] - fyn[q]);
          if (FLUX == 1 && !oE) g = 0.f;
          if (oE) {
            const float C = ch * ro;
            const float diff =
                t.kappa * (dxe[q] + dxw[q] + hvjp * (chjp * rjp - C) * c10 + hv * (C - chjm * rjm) * c11);
            const float gam = t.gamma ? t.gamma[ko] : t.gamma_s;
            g += diff - gam * Do * (C - pc0[q]) + C * Fe;
          }
          t.G3[ko] = g;
          const float inc = p.dt * (p.ab0 * pg1[q] + p.ab1 * pg2[q] + p.ab2 * g);
          float nh, nl;
          comp_update(RELOAD ? t.ch[ko] : chh[q][2], RELOAD ? t.cl[ko] : chl[q][2], inc, t.dp ? t.dp[ko] : t.dp_s,
                      nh, nl);
          t.chn[ko] = nh;
          t.cln[ko] = nl;
        }
      }
    }
    // update inputs of the next output row (J - 1)
    if (store_lane && J - 1 >= ry0 && J - 1 < ylast) {
      const int kn = gi + off[1];
#pragma unroll
      for (int q = 0; q < NT; q++) {
        pg1[q] = p.t[q].G1[kn];
        pg2[q] = p.t[q].G2[kn];
        pc0[q] = p.t[q].C0[kn];
      }
    }
  }
}

// rows per warp set by SWM_GB300_TRC_ROWS, 0 when unset
static int trc_rows_override() {
  const char *e = getenv("SWM_GB300_TRC_ROWS");
  if (e && atoi(e) >= 4 && atoi(e) <= 256) return atoi(e);
  return 0;
}

// Prefetch level of the tracer kernel (k_trc32's PF): 1 when the bytes one
// step moves (u, v, H, mask and eta 18 B per point, 32 B per tracer) exceed
// L2, so that every step reads its rows from DRAM.  SWM_GB300_TRC_PREFETCH=0/1
// forces it.
static int trc_prefetch(size_t points, int ntr) {
  const char *e = getenv("SWM_GB300_TRC_PREFETCH");
  if (e && (e[0] == '0' || e[0] == '1') && e[1] == 0) return e[0] - '0';
  return exceeds_l2((18.0 + 32.0 * ntr) * (double)points) ? 1 : 0;
}

template <int NT, int FLUX>
static void trc_launch_f(const TrcP &p, int S, cudaStream_t st) {
  const int nstrips = (p.nx + 27) / 28;
  const unsigned blocks = (unsigned)((long)nstrips * ((p.ny + 4 * S - 1) / (4 * S)));
  if (p.pf) k_trc32<NT, FLUX, 1><<<blocks, 128, 0, st>>>(p, S, nstrips);
  else k_trc32<NT, FLUX, 0><<<blocks, 128, 0, st>>>(p, S, nstrips);
}

template <int NT, int FLUX>
static int trc_resident_f(int pf) {
  int per_sm = 0, sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (pf) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trc32<NT, FLUX, 1>, 128, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trc32<NT, FLUX, 0>, 128, 0);
  return sms * (per_sm > 0 ? per_sm : 1);
}

template <int NT>
static void trc_launch_nt(const TrcP &p, int S, cudaStream_t st) {
  if (p.flux == 1) trc_launch_f<NT, 1>(p, S, st);
  else trc_launch_f<NT, 0>(p, S, st);
}

template <int NT>
static int trc_resident_nt(const TrcP &p) {
  return p.flux == 1 ? trc_resident_f<NT, 1>(p.pf) : trc_resident_f<NT, 0>(p.pf);
}

static void trc_launch(const TrcP &p, int S, cudaStream_t st) {
  switch (p.ntr) {
    case 1: trc_launch_nt<1>(p, S, st); break;
    case 2: trc_launch_nt<2>(p, S, st); break;
    case 3: trc_launch_nt<3>(p, S, st); break;
    default: trc_launch_nt<4>(p, S, st); break;
  }
}

// blocks of the tracer kernel resident on the whole GPU at once
static int trc_resident(const TrcP &p) {
  switch (p.ntr) {
    case 1: return trc_resident_nt<1>(p);
    case 2: return trc_resident_nt<2>(p);
    case 3: return trc_resident_nt<3>(p);
    default: return trc_resident_nt<4>(p);
  }
}

// Rows per warp, by timing the tracer step on this basin (the repeated step
// rewrites the next level and the newest increment only): TRC_ROWS, 32, 64
// and the lengths that make the grid one and two waves of resident blocks
// (the look-ahead costs 4 rows per warp, so longer warps do less of it, and
// a grid of whole waves has no partial last wave).
static int trc_tune_rows(swm_gpu_ctx *c, const TrcP &p) {
  const int env = trc_rows_override();
  if (env) return env;
  std::vector<int> cand = {TRC_ROWS, 32, 64};
  const int nstrips = (p.nx + 27) / 28, R = trc_resident(p);
  for (int waves = 1; waves <= 2; waves++) {
    const int per_strip = waves * R / nstrips;  // blocks of four row groups per strip
    if (per_strip < 1) continue;
    const int S = (p.ny + 4 * per_strip - 1) / (4 * per_strip);
    if (S >= 4 && S <= 256) cand.push_back(S);
  }
  std::sort(cand.begin(), cand.end());
  cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
  int best = TRC_ROWS;
  const int rc = march_pick_rows(c->stream, 3, cand, [&](int S) { trc_launch(p, S, c->stream); }, &best);
  return rc == SWM_GPU_OK ? best : TRC_ROWS;
}

__global__ void k_trc32_export(const float *ch, const float *cl, const double *D, double *out, size_t n, int conc) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double v = (double)ch[k] + (double)cl[k];
  out[k] = conc ? (D[k] != 0. ? v / D[k] : 0.) : v;
}

__global__ void k_f64_to_f32(const double *a, float *b, size_t n) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (float)a[k];
}

}  // namespace swm

struct Trc32State {
  std::vector<swm::Tracer32> t;
  int warp_rows = 0;  // rows per warp of the tracer kernel (0: not tuned yet)
  float *rows = nullptr;
  float *u = nullptr, *v = nullptr, *eta = nullptr;  // frozen-flow copies
  bool ready = false;
};

namespace swm {

static int t32_alloc(float **p, size_t n) {
  if (cudaMalloc((void **)p, n * sizeof(float)) != cudaSuccess) {
    set_error("trc32: cudaMalloc failed");
    return SWM_GPU_ENOMEM;
  }
  return SWM_GPU_OK;
}

#define T32TRY(x)                        \
  do {                                   \
    int rc_ = (x);                       \
    if (rc_ != SWM_GPU_OK) return rc_;   \
  } while (0)

static int upload_f32(swm_gpu_ctx *c, const std::vector<double> &h, float **dst) {
  std::vector<float> f(h.size());
  for (size_t k = 0; k < h.size(); k++) f[k] = (float)h[k];
  T32TRY(t32_alloc(dst, h.size()));
  SWM_CK(cudaMemcpyAsync(*dst, f.data(), f.size() * 4, cudaMemcpyHostToDevice, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}

static bool uniform_of(const std::vector<double> &a, double *v) {
  *v = a.empty() ? 0. : a[0];
  for (double x : a)
    if (x != *v) return false;
  return true;
}

bool trc32_active(const swm_gpu_ctx *c) { return c->cfg.path == SWM_PATH_FUSED_FP32C && !c->tracers.empty(); }

// FP32 copy of one tracer (called from trc_gpu_add with the FP64 host data)
int trc32_add(swm_gpu_ctx *c, const std::vector<double> &CH, const std::vector<double> &C0,
              const std::vector<double> &gamma, const std::vector<double> &impl, double kappa) {
  if (!c->trc32) c->trc32 = new Trc32State();
  Tracer32 T;
  const size_t n = c->n;
  std::vector<double> hi(n), lo(n);
  for (size_t k = 0; k < n; k++) {
    hi[k] = (double)(float)CH[k];
    lo[k] = CH[k] - hi[k];
  }
  for (int q = 0; q < 2; q++) {
    T32TRY(upload_f32(c, hi, &T.ch[q]));
    T32TRY(upload_f32(c, lo, &T.cl[q]));
  }
  for (int q = 0; q < 3; q++) {
    T32TRY(t32_alloc(&T.G[q], n));
    SWM_CK(cudaMemsetAsync(T.G[q], 0, n * 4, c->stream));
  }
  T32TRY(upload_f32(c, C0, &T.C0));
  double g;
  if (uniform_of(gamma, &g)) T.gamma_s = (float)g;
  else T32TRY(upload_f32(c, gamma, &T.gamma));
  std::vector<double> dp(n);
  for (size_t k = 0; k < n; k++) dp[k] = (impl[k] - 1.) / impl[k];
  double d;
  if (uniform_of(dp, &d)) T.dp_s = (float)d;
  else T32TRY(upload_f32(c, dp, &T.dp));
  T.kappa = (float)kappa;
  c->trc32->t.push_back(T);
  return SWM_GPU_OK;
}

// per-row factors and, for a frozen flow, FP32 copies of u, v, eta
int trc32_init(swm_gpu_ctx *c) {
  Trc32State *s = c->trc32;
  if (!s) return SWM_GPU_OK;
  T32TRY(fused_prepare(c));  // masks and depths of the FP32 path
  const HostGrid &g = c->hg;
  const double A = c->cfg.A, dL = g.dLambda, dT = g.dTheta;
  std::vector<double> rows((size_t)c->ny * RT_NR);
  for (int j = 0; j < c->ny; j++) {
    double *r = &rows[(size_t)j * RT_NR];
    double cE = g.cosl[GE][j], cU = g.cosl[GU][j], cV = g.cosl[GV][j];
    r[RT_RDL] = 1. / (A * dL * cE);
    r[RT_RDT] = 1. / (A * dT * cE);
    r[RT_CV] = cV;
    r[RT_D8] = 1. / (dL * dL) / (A * A) / cU / cE;
    r[RT_D10] = 1. / (dT * dT) / (A * A) / cE;
  }
  if (s->rows) cudaFree(s->rows);
  T32TRY(upload_f32(c, rows, &s->rows));
  if (c->cfg.frozen_flow) {
    const size_t n = c->n;
    unsigned nb = (unsigned)((n + 255) / 256);
    float **dst[3] = {&s->u, &s->v, &s->eta};
    const double *src[3] = {c->u[c->n0], c->v[c->n0], c->eta[c->n0]};
    for (int q = 0; q < 3; q++) {
      if (!*dst[q]) T32TRY(t32_alloc(dst[q], n));
      k_f64_to_f32<<<nb, 256, 0, c->stream>>>(src[q], *dst[q], n);
    }
    c->launches += 3;
  }
  s->ready = true;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

int trc32_step(swm_gpu_ctx *c, int64_t itt) {
  Trc32State *s = c->trc32;
  SWM_REQUIRE(s && s->ready, "tracers: call trc_gpu_init before stepping");
  int tstep = (int)(itt < 3 ? itt : 3);
  const double chi = c->cfg.ab_chi;
  double tab[4][3] = {{0, 0, 0}, {1., 0, 0}, {-0.5 - chi, 1.5 + chi, 0}, {5. / 12., -16. / 12., 23. / 12.}};
  TrcP p;
  memset(&p, 0, sizeof(p));
  p.nx = c->nx;
  p.ny = c->ny;
  p.nl = c->cfg.mode == SWM_MODE_NONLINEAR;
  p.flux = c->cfg.tracer_flux;
  p.dt = (float)c->cfg.dt;
  p.ab0 = (float)tab[tstep][0];
  p.ab1 = (float)tab[tstep][1];
  p.ab2 = (float)tab[tstep][2];
  const float *six[6];
  if (c->cfg.frozen_flow) {
    p.u = s->u; p.v = s->v; p.eta = s->eta;
  } else {
    fused_pair_level(c, six);  // the level the SWM step reads (TRC_timestep runs before SWM_advance)
    p.u = six[0]; p.v = six[2]; p.eta = six[4];
  }
  fused_static(c, &p.He, &p.mask16, &p.Fe);
  p.rows = s->rows;
  for (size_t t0 = 0; t0 < s->t.size(); t0 += TRC32_MAX) {
    p.ntr = (int)std::min(s->t.size() - t0, (size_t)TRC32_MAX);
    p.pf = trc_prefetch(c->n, p.ntr);
    for (int q = 0; q < p.ntr; q++) {
      const Tracer32 &T = s->t[t0 + q];
      auto &d = p.t[q];
      d.ch = T.ch[T.n0]; d.cl = T.cl[T.n0]; d.chn = T.ch[1 - T.n0]; d.cln = T.cl[1 - T.n0];
      d.G1 = T.G[T.g0]; d.G2 = T.G[(T.g0 + 1) % 3]; d.G3 = T.G[(T.g0 + 2) % 3];
      d.C0 = T.C0; d.gamma = T.gamma; d.dp = T.dp;
      d.gamma_s = T.gamma_s; d.dp_s = T.dp_s; d.kappa = T.kappa;
    }
    if (!s->warp_rows) s->warp_rows = trc_tune_rows(c, p);
    trc_launch(p, s->warp_rows, c->stream);
    c->launches++;
  }
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

void trc32_advance(swm_gpu_ctx *c) {
  for (auto &T : c->trc32->t) {
    T.n0 = 1 - T.n0;
    T.g0 = (T.g0 + 1) % 3;
  }
}

// CH (field 0) or C = CH / D (field 1) of tracer t into a device FP64 buffer
int trc32_export(swm_gpu_ctx *c, int t, int conc, double *dst) {
  Trc32State *s = c->trc32;
  SWM_REQUIRE(s && t >= 0 && t < (int)s->t.size(), "trc32: bad tracer");
  const Tracer32 &T = s->t[t];
  const size_t n = c->n;
  k_trc32_export<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(T.ch[T.n0], T.cl[T.n0], c->dev().D, dst, n,
                                                                     conc);
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

void trc32_free(swm_gpu_ctx *c) {
  Trc32State *s = c->trc32;
  if (!s) return;
  for (auto &T : s->t) {
    for (int q = 0; q < 2; q++) { cudaFree(T.ch[q]); cudaFree(T.cl[q]); }
    for (int q = 0; q < 3; q++) cudaFree(T.G[q]);
    cudaFree(T.C0); cudaFree(T.gamma); cudaFree(T.dp);
  }
  cudaFree(s->rows); cudaFree(s->u); cudaFree(s->v); cudaFree(s->eta);
  delete s;
  c->trc32 = nullptr;
}

}  // namespace swm
