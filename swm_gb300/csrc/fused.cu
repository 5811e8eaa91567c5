// fused.cu -- one-kernel-per-step SWM update (FULLY_NONLINEAR,
// LINEARISED_STATE_OF_REST and no-linearisation modes).
//
// A CTA owns a TX x TY tile of cells.  It stages u, v, eta, the land/ocean
// mask code and the depth for the tile plus an H-cell halo (H = 1 for the
// reference's Laplacian-type stress, 2 for the biharmonic extension) in
// shared memory, rebuilds every per-step diagnostic the reference keeps in
// global arrays (D, Du/Dv/Dh, mass fluxes, vorticity, PV, Bernoulli,
// P_lambda-lambda / P_lambda-theta) inside the tile, and writes only the new
// state and the newest Adams-Bashforth increment.  Per cell and step the
// kernel therefore moves the state in and out once, reads the two older
// increments and writes the newest one -- the algorithmic minimum.
//
// T = double: the FP64 fused path.  (The FP32 compensated path is the row
// marching kernel of march.cu.)
//
// Arithmetic follows the reference formulas (swm_nonlinear_timestep_module.f90
// :182-449, swm_lateralmixing_module.f90:66-240, time_integration_module.f90
// :74-112) with divisions by grid metrics replaced by per-row reciprocals, so
// results agree with the FP64 restatement to rounding, not bit for bit.
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>
#include "ctx.h"
#include "fused32.h"

namespace swm {

enum {
  R_CE, R_CV, R_CU, R_FH, R_RE_DL, R_RE_DT, R_RU_DL, R_RV_DL, R_RH_DL, R_INV_CH,
  R_PC0, R_HC0, R_TE, R_TH, R_TU, R_TV, R_NR
};

template <typename T>
struct FP {
  int nx, ny, mode, mix, qbf, barotropic, has_F, impl_uniform, gsq_uniform, wind_x, wind_y, wind_rows, tstep;
  T dt, G, minD, lbc, q1, ts_rho, Ah, bih, eps;
  T ab0, ab1, ab2;
  T impl_s[3], gsq_s[2];
  const uint8_t *mc;
  const T *He, *rows, *Hu, *Hv;
  const T *impl[3], *gsq[2];
  const T *Fx, *Fy, *Fe;
  const T *wx, *wy;
  const T *u0, *v0, *e0;
  T *u1, *v1, *e1;
  const T *Gu1, *Gu2, *Gv1, *Gv2, *Ge1, *Ge2;
  T *Gu3, *Gv3, *Ge3;
};

constexpr int TX = 32, TY = 8, NT = TX * TY;

__device__ __forceinline__ int wrapi(int g, int n) {
  if (g < 0) g += n;
  if (g >= n) g -= n;
  if (g >= n) g -= n;
  return g;
}

template <typename T>
__device__ __forceinline__ T recip_cnt(int c) {
  // 1 / max(c, 1) for the mask-normalised interpolation weights
  return c <= 1 ? T(1) : (c == 2 ? T(0.5) : (c == 3 ? T(1) / T(3) : T(0.25)));
}

template <typename T, int HALO>
__global__ void __launch_bounds__(NT) k_fused(FP<T> p) {
  constexpr int W = TX + 2 * HALO, HH = TY + 2 * HALO, NS = W * HH;
  __shared__ T sU[NS], sV[NS], sE[NS], sD[NS], sMU[NS], sMV[NS], sPOT[NS], sB[NS], sPLL[NS], sPLT[NS];
  __shared__ T sLU[HALO == 2 ? NS : 1], sLV[HALO == 2 ? NS : 1];
  __shared__ uint8_t sM[NS];
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int nx = p.nx, ny = p.ny;
  const bool nl = p.mode == SWM_MODE_NONLINEAR;
  auto S = [](int i, int j) { return (j + HALO) * W + (i + HALO); };
  auto row = [&](int j) { return p.rows + (size_t)wrapi(j0 + j, ny) * R_NR; };

  // ---- phase A: stage state, mask and thickness ----------------------
  for (int q = tid; q < NS; q += NT) {
    int ti = q % W - HALO, tj = q / W - HALO;
    int gi = wrapi(i0 + ti, nx), gj = wrapi(j0 + tj, ny);
    size_t k = (size_t)gi + (size_t)nx * gj;
    uint8_t m = p.mc[k];
    T e = p.e0[k], he = p.He[k];
    sM[q] = m;
    sU[q] = p.u0[k];
    sV[q] = p.v0[k];
    sE[q] = e;
    // computeD: D = eta + H on ocean eta (FULLY_NONLINEAR, land keeps 1),
    // else the eta-grid depth
    sD[q] = nl ? ((m & 8) ? e + he : T(1)) : he;
  }
  __syncthreads();

  auto oH = [&](int q) { return sM[q] & 1; };
  auto oU = [&](int q) { return (sM[q] >> 1) & 1; };
  auto oV = [&](int q) { return (sM[q] >> 2) & 1; };
  auto oE = [&](int q) { return (sM[q] >> 3) & 1; };
  auto Du_at = [&](int q) {  // eta2u_noland of D
    int a = oE(q), b = oE(q - 1);
    return (T(a) * sD[q] + T(b) * sD[q - 1]) * recip_cnt<T>(a + b);
  };
  auto Dv_at = [&](int q) {
    int a = oE(q), b = oE(q - W);
    return (T(a) * sD[q] + T(b) * sD[q - W]) * recip_cnt<T>(a + b);
  };
  auto Dh_at = [&](int q) {  // eta2H_noland: (i,j),(i-1,j-1),(i-1,j),(i,j-1)
    int a = oE(q), b = oE(q - W - 1), c = oE(q - 1), d = oE(q - W);
    return (T(a) * sD[q] + T(b) * sD[q - W - 1] + T(c) * sD[q - 1] + T(d) * sD[q - W]) * recip_cnt<T>(a + b + c + d);
  };
  auto inner = [&](int ti, int tj, int lo, int hi_) {
    return ti >= -HALO + lo && ti < TX + HALO - hi_ && tj >= -HALO + lo && tj < TY + HALO - hi_;
  };

  // P tensor of the Laplacian-type stress at eta (pll) and H (plt) points for
  // the velocity pair (a, b) = (u-like, v-like), weights on (weighted) or 1
  auto p_tensor = [&](const T *a, const T *b, T Ah, bool weighted, T *outL, T *outT) {
    for (int q = tid; q < NS; q += NT) {
      int ti = q % W - HALO, tj = q / W - HALO;
      T pl = T(0), pt = T(0);
      if (ti < TX + HALO - 1 && tj < TY + HALO - 1 && oE(q)) {  // needs (i+1, j), (i, j+1)
        const T *r = row(tj);
        int ov = oV(q), ovp = oV(q + W);
        T tE = r[R_TE] * recip_cnt<T>(ov + ovp);  // counts 0..2: exactly the division
        T c0 = Ah * r[R_PC0];
        T c1 = Ah * (p.q1 + T(ovp) * tE);
        T c2 = Ah * (-p.q1 + T(ov) * tE);
        pl = (weighted ? sD[q] : T(1)) * (c0 * (a[q + 1] - a[q]) + c1 * b[q + W] + c2 * b[q]);
      }
      if (ti > -HALO && tj > -HALO && oH(q)) {  // needs (i-1, j), (i, j-1)
        const T *r = row(tj);
        int ou = oU(q), oum = oU(q - W);
        T tH = r[R_TH] * recip_cnt<T>(ou + oum);
        T c0 = Ah * r[R_HC0];
        T c1 = -Ah * (p.q1 + T(ou) * tH);
        T c2 = -Ah * (-p.q1 + T(oum) * tH);
        pt = (weighted ? Dh_at(q) : T(1)) * (c0 * (b[q] - b[q - 1]) + c1 * a[q] + c2 * a[q - W]);
      }
      outL[q] = pl;
      outT[q] = pt;
    }
  };
  // divergence of P onto u and v points (compute_uv); unit thickness or D
  auto lat_u = [&](int q, int tj, bool weighted) {
    const T *r = row(tj);
    int o = oH(q) + oH(q + W);
    T t2 = T(2) * r[R_TU] * recip_cnt<T>(o);
    T m0 = -r[R_RU_DL], m1 = -(p.q1 - t2), m2 = p.q1 + t2;
    T s = m0 * (sPLL[q] - sPLL[q - 1]) + m1 * sPLT[q + W] + m2 * sPLT[q];
    return weighted ? s / Du_at(q) : s;
  };
  auto lat_v = [&](int q, int tj, bool weighted) {
    const T *r = row(tj);
    int o = oE(q) + oE(q - W);
    T t2 = T(2) * r[R_TV] * recip_cnt<T>(o);
    T m0 = -r[R_RV_DL], m1 = p.q1 - t2, m2 = -(p.q1 + t2);
    T s = m0 * (sPLT[q + 1] - sPLT[q]) + m1 * sPLL[q] + m2 * sPLL[q - W];
    return weighted ? s / Dv_at(q) : s;
  };

  if (p.mix == 2) {
    // biharmonic extension: first pass with unit thickness and Ah = 1
    p_tensor(sU, sV, T(1), false, sPLL, sPLT);
    __syncthreads();
    for (int q = tid; q < NS; q += NT) {
      int ti = q % W - HALO, tj = q / W - HALO;
      bool ok = inner(ti, tj, 1, 1);
      sLU[q] = (ok && oU(q)) ? lat_u(q, tj, false) : T(0);
      sLV[q] = (ok && oV(q)) ? lat_v(q, tj, false) : T(0);
    }
    __syncthreads();
  }

  // ---- phase B: mass fluxes, PV, Bernoulli, P tensor -------------------
  for (int q = tid; q < NS; q += NT) {
    int ti = q % W - HALO, tj = q / W - HALO;
    bool lo_ok = ti > -HALO && tj > -HALO;
    bool hi_ok = ti < TX + HALO - 1 && tj < TY + HALO - 1;
    sMU[q] = (ti > -HALO && oU(q)) ? Du_at(q) * sU[q] : T(0);
    sMV[q] = (tj > -HALO && oV(q)) ? Dv_at(q) * sV[q] : T(0);
    T pot = T(0);
    if (lo_ok && p.mode != SWM_MODE_NONE) {
      const T *r = row(tj);
      T zeta = T(0);
      if (nl) {
        T bc = oH(q) ? T(1) : p.lbc;
        T dvdx = (oV(q - 1) + oV(q) == 0) ? T(0) : bc * r[R_RH_DL] * (sV[q] - sV[q - 1]);
        T dudy = (oU(q) + oU(q - W) == 0) ? T(0) : bc * p.q1 * (r[R_CU] * sU[q] - row(tj - 1)[R_CU] * sU[q - W]);
        zeta = dvdx - dudy * r[R_INV_CH];
      }
      T pD = Dh_at(q);
      pD = pD > p.eps ? pD : p.eps;
      pot = (r[R_FH] + zeta) / pD;
    }
    sPOT[q] = pot;
    T b = T(0);
    if (hi_ok && oE(q) && p.mode != SWM_MODE_NONE) {
      b = p.G * sE[q];
      if (nl) {
        T a = T(0.5) * (sU[q + 1] * sU[q + 1]) + T(0.5) * (sU[q] * sU[q]);
        T c = T(0.5) * (sV[q + W] * sV[q + W]) + T(0.5) * (sV[q] * sV[q]);
        b = (a + c) * T(0.5) + b;
      }
    }
    sB[q] = b;
  }
  if (p.mix == 1) p_tensor(sU, sV, p.Ah, true, sPLL, sPLT);
  if (p.mix == 2) {
    __syncthreads();  // lat_u/lat_v of the first pass read sPLL/sPLT
    p_tensor(sLU, sLV, -p.bih, true, sPLL, sPLT);
  }
  __syncthreads();

  // ---- phase C: tendencies and Adams-Bashforth update (interior) ------
  for (int q0 = tid; q0 < TX * TY; q0 += NT) {
    int ti = q0 % TX, tj = q0 / TX;
    int gi = i0 + ti, gj = j0 + tj;
    if (gi >= nx || gj >= ny) continue;
    size_t k = (size_t)gi + (size_t)nx * gj;
    int q = S(ti, tj);
    const T *r = row(tj);
    T ge = T(0), gu = T(0), gv = T(0);
    if (oE(q)) {
      T cvp = row(tj + 1)[R_CV], cv = r[R_CV];
      ge = -(sMU[q + 1] - sMU[q]) * r[R_RE_DL] - (sMV[q + W] * cvp - sMV[q] * cv) * r[R_RE_DT];
      if (p.has_F) ge = ge + p.Fe[k];
    }
    if (oU(q)) {
      T pv = T(0.5) * sPOT[q + W] + T(0.5) * sPOT[q];
      T mv = T(0.25) * sMV[q + W] + T(0.25) * sMV[q - 1] + T(0.25) * sMV[q - 1 + W] + T(0.25) * sMV[q];
      T g = pv * mv - (sB[q] - sB[q - 1]) * r[R_RU_DL];
      if (p.qbf) {
        T vb = T(0.25) * sV[q + W] + T(0.25) * sV[q - 1] + T(0.25) * sV[q - 1 + W] + T(0.25) * sV[q];
        T gs = p.gsq_uniform ? p.gsq_s[0] : p.gsq[0][k];
        T f = gs * sqrt(sU[q] * sU[q] + vb * vb) * sU[q];
        if (p.barotropic) f = f / p.Hu[k];
        g = g - f;
      }
      if (p.mix) g = g + lat_u(q, tj, true);
      if (p.has_F) g = g + p.Fx[k];
      if (p.wind_x) g = g + p.ts_rho * (p.wind_rows ? p.wx[gj] : p.wx[k]) / (nl ? Du_at(q) : T(1));
      gu = g;
    }
    if (oV(q)) {
      T pv = T(0.5) * sPOT[q + 1] + T(0.5) * sPOT[q];
      T mu = T(0.25) * sMU[q + 1] + T(0.25) * sMU[q - W] + T(0.25) * sMU[q] + T(0.25) * sMU[q + 1 - W];
      T g = -pv * mu - (sB[q] - sB[q - W]) * p.q1;
      if (p.qbf) {
        T ub = T(0.25) * sU[q + 1] + T(0.25) * sU[q - W] + T(0.25) * sU[q] + T(0.25) * sU[q + 1 - W];
        T gs = p.gsq_uniform ? p.gsq_s[1] : p.gsq[1][k];
        T f = gs * sqrt(sV[q] * sV[q] + ub * ub) * sV[q];
        if (p.barotropic) f = f / p.Hv[k];
        g = g - f;
      }
      if (p.mix) g = g + lat_v(q, tj, true);
      if (p.has_F) g = g + p.Fy[k];
      if (p.wind_y) g = g + p.ts_rho * (p.wind_rows ? p.wy[gj] : p.wy[k]) / (nl ? Dv_at(q) : T(1));
      gv = g;
    }
    p.Ge3[k] = ge;
    p.Gu3[k] = gu;
    p.Gv3[k] = gv;
    T ie = p.impl_uniform ? p.impl_s[2] : p.impl[2][k];
    T iu = p.impl_uniform ? p.impl_s[0] : p.impl[0][k];
    T iv = p.impl_uniform ? p.impl_s[1] : p.impl[1][k];
    T ince = p.dt * (p.ab0 * p.Ge1[k] + p.ab1 * p.Ge2[k] + p.ab2 * ge);
    T incu = p.dt * (p.ab0 * p.Gu1[k] + p.ab1 * p.Gu2[k] + p.ab2 * gu);
    T incv = p.dt * (p.ab0 * p.Gv1[k] + p.ab1 * p.Gv2[k] + p.ab2 * gv);
    T lim = p.minD - p.He[k];
    T e = (sE[q] + ince) / ie;
    if (nl && e < lim) e = lim;
    p.e1[k] = e;
    p.u1[k] = (sU[q] + incu) / iu;
    p.v1[k] = (sV[q] + incv) / iv;
  }
}

// FP64 <-> FP32 hi/lo conversions
__global__ void k_split(const double *src, float *hi, float *lo, size_t n) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double x = src[k];
  float h = (float)x;
  hi[k] = h;
  lo[k] = (float)(x - (double)h);
}
__global__ void k_join(const float *hi, const float *lo, double *dst, size_t n) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  dst[k] = (double)hi[k] + (lo ? (double)lo[k] : 0.);
}
__global__ void k_to_f32(const double *src, float *dst, size_t n) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = (float)src[k];
}

struct P32;
std::vector<double> fp32c_rows(const swm_gpu_ctx *c);
}  // namespace swm

using namespace swm;

struct FusedState {
  bool ready = false;
  bool comp = false;
  // FP32 pair state and increments (FP32C path)
  float *uh[2] = {}, *ul[2] = {}, *vh[2] = {}, *vl[2] = {}, *eh[2] = {}, *el[2] = {};
  float *Gu[3] = {}, *Gv[3] = {}, *Ge[3] = {};
  // static inputs
  uint8_t *mc = nullptr;
  void *He = nullptr, *rows = nullptr, *Hu = nullptr, *Hv = nullptr;
  void *impl[3] = {}, *gsq[2] = {}, *F[3] = {}, *wx = nullptr, *wy = nullptr;
  void *rows32c = nullptr;
  uint16_t *mask16 = nullptr;
  std::vector<uint16_t> m16h;  // host copy of mask16 (the step kernel's tiles are cut from it)
  void *dp[3] = {};
  double dp_s[3] = {0, 0, 0};
  bool impl_uniform = true, gsq_uniform = true, has_F = false, wind_rows = false;
  int wind_x = 0, wind_y = 0;
  double impl_s[3] = {1, 1, 1}, gsq_s[2] = {0, 0};
  int n0 = 0, g0 = 0;  // FP32C level / ring indices
  // forcing that changes every step (LINEARISED_MEAN_STATE terms, oscillating
  // streams): F = Fc + this step's part, written before the step kernel;
  // the per-step relative vorticity and energy term of the mean state
  bool lin_mean = false, dyn_F = false;
  void *Fc[3] = {};
  double *ms_zeta = nullptr, *ms_ex = nullptr;
};

namespace swm {

// 16 bytes more than asked: the step kernel's row copies move whole 16-byte
// words and may read up to 12 bytes past a field's last element
static int dmalloc(void **p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes + 16);
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return SWM_GPU_ENOMEM;
  }
  return SWM_GPU_OK;
}

#define FTRY(x)                          \
  do {                                   \
    int rc_ = (x);                       \
    if (rc_ != SWM_GPU_OK) return rc_;   \
  } while (0)

// device copy of a host FP64 array in the path's precision
static int upload_t(swm_gpu_ctx *c, bool f32, const double *host, size_t count, void **dst) {
  size_t es = f32 ? 4 : 8;
  FTRY(dmalloc(dst, count * es));
  if (f32) {
    std::vector<float> t(count);
    for (size_t q = 0; q < count; q++) t[q] = (float)host[q];
    SWM_CK(cudaMemcpy(*dst, t.data(), count * 4, cudaMemcpyHostToDevice));
  } else {
    SWM_CK(cudaMemcpy(*dst, host, count * 8, cudaMemcpyHostToDevice));
  }
  return SWM_GPU_OK;
}

static bool uniform(const std::vector<double> &v, double *val) {
  for (size_t q = 1; q < v.size(); q++)
    if (v[q] != v[0]) return false;
  *val = v.empty() ? 0. : v[0];
  return true;
}

static void download(swm_gpu_ctx *c, const double *dev, std::vector<double> &out) {
  out.resize(c->n);
  cudaMemcpyAsync(out.data(), dev, c->n * 8, cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
}

// Builds the static inputs of the fused kernel once the model is initialised.
int fused_prepare(swm_gpu_ctx *c) {
  FusedState *f = c->fused;
  if (f && f->ready) return SWM_GPU_OK;
  const swm_gpu_config &cf = c->cfg;
  if (!f) f = c->fused = new FusedState();
  f->lin_mean = cf.mode == SWM_MODE_LIN_MEAN;
  bool f32 = cf.path == SWM_PATH_FUSED_FP32C;
  f->comp = f32;
  size_t n = c->n;
  int ny = c->ny;
  const HostGrid &g = c->hg;
  // mask code: bit0 H, bit1 u, bit2 v, bit3 eta
  std::vector<uint8_t> mc(n);
  for (size_t k = 0; k < n; k++)
    mc[k] = (uint8_t)(g.ocean[GH][k] | (g.ocean[GU][k] << 1) | (g.ocean[GV][k] << 2) | (g.ocean[GE][k] << 3));
  FTRY(dmalloc((void **)&f->mc, n));
  SWM_CK(cudaMemcpy(f->mc, mc.data(), n, cudaMemcpyHostToDevice));
  // per-row metric factors, from the FP64 grid
  std::vector<double> rows((size_t)ny * R_NR);
  double A = cf.A, dL = g.dLambda, dT = g.dTheta;
  for (int j = 0; j < ny; j++) {
    double *r = &rows[(size_t)j * R_NR];
    double cE = g.cosl[GE][j], cV = g.cosl[GV][j], cU = g.cosl[GU][j], cH = g.cosl[GH][j];
    r[R_CE] = cE;
    r[R_CV] = cV;
    r[R_CU] = cU;
    r[R_FH] = g.f[GH][j];
    r[R_RE_DL] = 1. / (A * cE * dL);
    r[R_RE_DT] = 1. / (A * cE * dT);
    r[R_RU_DL] = 1. / (A * cU * dL);
    r[R_RV_DL] = 1. / (A * cV * dL);
    r[R_RH_DL] = 1. / (A * cH * dL);
    r[R_INV_CH] = 1. / cH;
    r[R_PC0] = -1. / (dL * A * cE);
    r[R_HC0] = -1. / (dL * A * cH);
    r[R_TE] = g.tanl[GE][j] / A;
    r[R_TH] = g.tanl[GH][j] / A;
    r[R_TU] = g.tanl[GU][j] / A;
    r[R_TV] = g.tanl[GV][j] / A;
  }
  FTRY(upload_t(c, f32, rows.data(), rows.size(), &f->rows));
  // depths (after computeD at itt = 0)
  std::vector<double> tmp;
  download(c, c->d_H[GE], tmp);
  FTRY(upload_t(c, f32, tmp.data(), n, &f->He));
  download(c, c->d_H[GU], tmp);
  FTRY(upload_t(c, f32, tmp.data(), n, &f->Hu));
  download(c, c->d_H[GV], tmp);
  FTRY(upload_t(c, f32, tmp.data(), n, &f->Hv));
  // damping
  f->impl_uniform = true;
  for (int q = 0; q < 3; q++) f->impl_uniform = f->impl_uniform && uniform(g.impl[q], &f->impl_s[q]);
  if (!f->impl_uniform)
    for (int q = 0; q < 3; q++) FTRY(upload_t(c, f32, g.impl[q].data(), n, &f->impl[q]));
  f->gsq_uniform = uniform(g.gsq[0], &f->gsq_s[0]) && uniform(g.gsq[1], &f->gsq_s[1]);
  if (!f->gsq_uniform)
    for (int q = 0; q < 2; q++) FTRY(upload_t(c, f32, g.gsq[q].data(), n, &f->gsq[q]));
  // forcing: constant part from the forcing arrays, NL wind recomputed in the kernel
  std::vector<double> Fh[3];
  f->has_F = false;
  for (int q = 0; q < 3; q++) {
    download(c, c->Fc[q], Fh[q]);
    for (double x : Fh[q]) f->has_F = f->has_F || x != 0.;
  }
  for (const Stream &s : c->streams) {
    if (s.is_const) continue;
    bool nl_wind = s.type == SWM_FRC_WIND && cf.mode == SWM_MODE_NONLINEAR &&
                   (s.comp == SWM_CMP_ZONAL || s.comp == SWM_CMP_MERID);
    if (!nl_wind) {  // added to the forcing fields every step (dyn_forcing)
      f->dyn_F = true;
      continue;
    }
    std::vector<double> d;
    download(c, s.d1, d);
    bool rowwise = true;
    for (int j = 0; j < ny && rowwise; j++)
      for (int i = 1; i < c->nx; i++)
        if (d[i + (size_t)c->nx * j] != d[(size_t)c->nx * j]) { rowwise = false; break; }
    int &flag = s.comp == SWM_CMP_ZONAL ? f->wind_x : f->wind_y;
    void *&dst = s.comp == SWM_CMP_ZONAL ? f->wx : f->wy;
    SWM_REQUIRE(!flag, "fused paths: one wind stress stream per component");
    flag = 1;
    if (rowwise) {
      std::vector<double> prof(ny);
      for (int j = 0; j < ny; j++) prof[j] = d[(size_t)c->nx * j];
      FTRY(upload_t(c, f32, prof.data(), ny, &dst));
    } else {
      FTRY(upload_t(c, f32, d.data(), n, &dst));
    }
    f->wind_rows = rowwise;
  }
  if (f->wind_x && f->wind_y) SWM_REQUIRE(f->wind_rows, "fused paths: two wind components must both be row profiles");
  f->dyn_F = f->dyn_F || f->lin_mean;
  if (f->dyn_F) {
    // every step writes F = Fc + its own part (dyn_forcing)
    f->has_F = true;
    for (int q = 0; q < 3; q++) FTRY(upload_t(c, f32, Fh[q].data(), n, &f->Fc[q]));
  }
  if (f->lin_mean) {
    FTRY(dmalloc((void **)&f->ms_zeta, n * 8));
    FTRY(dmalloc((void **)&f->ms_ex, n * 8));
  }
  if (f->has_F)
    for (int q = 0; q < 3; q++) FTRY(upload_t(c, f32, Fh[q].data(), n, &f->F[q]));
  if (f32) {
    const std::vector<float> rec = fp32c_records(c);
    FTRY(dmalloc(&f->rows32c, rec.size() * sizeof(float)));
    SWM_CK(cudaMemcpy(f->rows32c, rec.data(), rec.size() * sizeof(float), cudaMemcpyHostToDevice));
    // mask word with the x-neighbours' bits (bits 4-7: i-1, 8-11: i+1)
    std::vector<uint16_t> m16(n);
    int nx = c->nx;
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        size_t k = i + (size_t)nx * j;
        size_t kl = (i == 0 ? nx - 1 : i - 1) + (size_t)nx * j, kr = (i + 1 == nx ? 0 : i + 1) + (size_t)nx * j;
        m16[k] = (uint16_t)(mc[k] | (mc[kl] << 4) | (mc[kr] << 8));
      }
    FTRY(dmalloc((void **)&f->mask16, n * 2));
    SWM_CK(cudaMemcpy(f->mask16, m16.data(), n * 2, cudaMemcpyHostToDevice));
    f->m16h = std::move(m16);
    // implicit damping as the removed fraction dt*gamma/(1 + dt*gamma)
    for (int q = 0; q < 3; q++) f->dp_s[q] = (f->impl_s[q] - 1.) / f->impl_s[q];
    if (!f->impl_uniform)
      for (int q = 0; q < 3; q++) {
        std::vector<double> dpq(n);
        for (size_t k = 0; k < n; k++) dpq[k] = (g.impl[q][k] - 1.) / g.impl[q][k];
        FTRY(upload_t(c, true, dpq.data(), n, &f->dp[q]));
      }
    for (int q = 0; q < 2; q++) {
      FTRY(dmalloc((void **)&f->uh[q], n * 4)); FTRY(dmalloc((void **)&f->ul[q], n * 4));
      FTRY(dmalloc((void **)&f->vh[q], n * 4)); FTRY(dmalloc((void **)&f->vl[q], n * 4));
      FTRY(dmalloc((void **)&f->eh[q], n * 4)); FTRY(dmalloc((void **)&f->el[q], n * 4));
    }
    for (int q = 0; q < 3; q++) {
      FTRY(dmalloc((void **)&f->Gu[q], n * 4)); FTRY(dmalloc((void **)&f->Gv[q], n * 4));
      FTRY(dmalloc((void **)&f->Ge[q], n * 4));
    }
  }
  f->ready = true;
  FTRY(fused_load_state(c));
  if (f32 && !c->march_rows) {
    // rows per warp strip, by timing the step on this basin (the repeated
    // step rewrites level N0p1 and slot 3 only, which the first real step
    // rewrites again)
    P32 p;
    make_p32(c, 3, p);
    FTRY(march_autotune(c, p, f->m16h.data()));
  }
  return SWM_GPU_OK;
}

// FP64 state and increments -> FP32 pair buffers (FP32C path)
int fused_load_state(swm_gpu_ctx *c) {
  FusedState *f = c->fused;
  if (!f || !f->ready || !f->comp) return SWM_GPU_OK;
  size_t n = c->n;
  unsigned nb = (unsigned)((n + 255) / 256);
  f->n0 = c->n0;
  f->g0 = c->g0;
  for (int q = 0; q < 2; q++) {
    k_split<<<nb, 256, 0, c->stream>>>(c->u[q], f->uh[q], f->ul[q], n);
    k_split<<<nb, 256, 0, c->stream>>>(c->v[q], f->vh[q], f->vl[q], n);
    k_split<<<nb, 256, 0, c->stream>>>(c->eta[q], f->eh[q], f->el[q], n);
  }
  for (int q = 0; q < 3; q++) {
    k_to_f32<<<nb, 256, 0, c->stream>>>(c->Gu[q], f->Gu[q], n);
    k_to_f32<<<nb, 256, 0, c->stream>>>(c->Gv[q], f->Gv[q], n);
    k_to_f32<<<nb, 256, 0, c->stream>>>(c->Ge[q], f->Ge[q], n);
  }
  c->launches += 15;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// FP32 pair state -> FP64 buffers of the current level (host reads, diagnostics)
int fused_sync_state(swm_gpu_ctx *c) {
  FusedState *f = c->fused;
  if (!f || !f->ready || !f->comp) return SWM_GPU_OK;
  size_t n = c->n;
  unsigned nb = (unsigned)((n + 255) / 256);
  int a = f->n0;
  k_join<<<nb, 256, 0, c->stream>>>(f->uh[a], f->ul[a], c->u[c->n0], n);
  k_join<<<nb, 256, 0, c->stream>>>(f->vh[a], f->vl[a], c->v[c->n0], n);
  k_join<<<nb, 256, 0, c->stream>>>(f->eh[a], f->el[a], c->eta[c->n0], n);
  int g2 = (f->g0 + 1) % 3, cg2 = (c->g0 + 1) % 3;
  k_join<<<nb, 256, 0, c->stream>>>(f->Gu[g2], nullptr, c->Gu[cg2], n);
  k_join<<<nb, 256, 0, c->stream>>>(f->Gv[g2], nullptr, c->Gv[cg2], n);
  k_join<<<nb, 256, 0, c->stream>>>(f->Ge[g2], nullptr, c->Ge[cg2], n);
  c->launches += 6;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

template <typename T>
static void fill_common(swm_gpu_ctx *c, FP<T> &p, int64_t itt) {
  const swm_gpu_config &cf = c->cfg;
  FusedState *f = c->fused;
  p.nx = c->nx;
  p.ny = c->ny;
  p.mode = cf.mode;
  p.mix = cf.lateral_mixing ? (cf.mixing_kind == SWM_MIX_BIHARMONIC ? 2 : 1) : 0;
  p.qbf = cf.quadratic_friction;
  p.barotropic = cf.barotropic;
  p.has_F = f->has_F;
  p.impl_uniform = f->impl_uniform;
  p.gsq_uniform = f->gsq_uniform;
  p.wind_x = f->wind_x;
  p.wind_y = f->wind_y;
  p.wind_rows = f->wind_rows;
  int tstep = (int)(itt < 3 ? itt : 3);
  p.tstep = tstep;
  double chi = cf.ab_chi;
  double tab[4][3] = {{0, 0, 0}, {1., 0, 0}, {-0.5 - chi, 1.5 + chi, 0}, {5. / 12., -16. / 12., 23. / 12.}};
  p.ab0 = (T)tab[tstep][0];
  p.ab1 = (T)tab[tstep][1];
  p.ab2 = (T)tab[tstep][2];
  p.dt = (T)cf.dt;
  // without a linearisation define EDens stays 0: no pressure gradient
  // (swm_nonlinear_timestep_module.f90:291-305)
  p.G = cf.mode == SWM_MODE_NONE ? (T)0 : (T)cf.G;
  p.minD = (T)cf.minD;
  p.lbc = (T)cf.lbc;
  p.q1 = (T)(1. / (cf.A * c->hg.dTheta));
  p.ts_rho = (T)(cf.tau_scale / cf.RHO0);
  p.Ah = (T)cf.Ah;
  p.bih = (T)cf.bih;
  p.eps = sizeof(T) == 8 ? (T)2.220446049250313e-16 : (T)1.1920929e-07;
  for (int q = 0; q < 3; q++) p.impl_s[q] = (T)f->impl_s[q];
  for (int q = 0; q < 2; q++) p.gsq_s[q] = (T)f->gsq_s[q];
  p.mc = f->mc;
  p.He = (const T *)f->He;
  p.rows = (const T *)f->rows;
  p.Hu = (const T *)f->Hu;
  p.Hv = (const T *)f->Hv;
  for (int q = 0; q < 3; q++) p.impl[q] = (const T *)f->impl[q];
  for (int q = 0; q < 2; q++) p.gsq[q] = (const T *)f->gsq[q];
  p.Fx = (const T *)f->F[0];
  p.Fy = (const T *)f->F[1];
  p.Fe = (const T *)f->F[2];
  p.wx = (const T *)f->wx;
  p.wy = (const T *)f->wy;
}

template <typename T>
static void launch_fused(swm_gpu_ctx *c, const FP<T> &p) {
  dim3 grid((c->nx + TX - 1) / TX, (c->ny + TY - 1) / TY);
  if (p.mix == 2) k_fused<T, 2><<<grid, NT, 0, c->stream>>>(p);
  else k_fused<T, 1><<<grid, NT, 0, c->stream>>>(p);
  c->launches++;
}


// parameter block of the FP32 step kernel for step itt from the context's
// current level and ring offsets
void make_p32(const swm_gpu_ctx *c, int64_t itt, P32 &p) {
  const swm_gpu_config &cf = c->cfg;
  const FusedState *f = c->fused;
  memset(&p, 0, sizeof(p));
  p.nx = c->nx;
  p.ny = c->ny;
  p.nl = cf.mode == SWM_MODE_NONLINEAR;
  p.has_mode = cf.mode != SWM_MODE_NONE;
  p.mix = cf.lateral_mixing ? (cf.mixing_kind == SWM_MIX_BIHARMONIC ? 2 : 1) : 0;
  p.qbf = cf.quadratic_friction;
  p.barotropic = cf.barotropic;
  p.has_F = f->has_F;
  p.impl_uniform = f->impl_uniform;
  p.gsq_uniform = f->gsq_uniform;
  p.wind_x = f->wind_x;
  p.wind_y = f->wind_y;
  p.wind_rows = f->wind_rows;
  int tstep = (int)(itt < 3 ? itt : 3);
  double chi = cf.ab_chi;
  double tab[4][3] = {{0, 0, 0}, {1., 0, 0}, {-0.5 - chi, 1.5 + chi, 0}, {5. / 12., -16. / 12., 23. / 12.}};
  p.ab0 = (float)tab[tstep][0];
  p.ab1 = (float)tab[tstep][1];
  p.ab2 = (float)tab[tstep][2];
  p.dt = (float)cf.dt;
  p.G = cf.mode == SWM_MODE_NONE ? 0.f : (float)cf.G;  // EDens stays 0 without a mode define
  p.minD = (float)cf.minD;
  p.lbc = (float)cf.lbc;
  p.q1 = (float)(1. / (cf.A * c->hg.dTheta));
  p.ts_rho = (float)(cf.tau_scale / cf.RHO0);
  p.Ah = (float)cf.Ah;
  p.bih = (float)cf.bih;
  for (int q = 0; q < 3; q++) {
    p.impl_s[q] = (float)f->impl_s[q];
    p.dp_s[q] = (float)f->dp_s[q];
    p.dp[q] = (const float *)f->dp[q];
  }
  for (int q = 0; q < 2; q++) p.gsq_s[q] = (float)f->gsq_s[q];
  p.mask16 = f->mask16;
  p.He = (const float *)f->He;
  p.rec = (const float4 *)f->rows32c;
  p.Hu = (const float *)f->Hu;
  p.Hv = (const float *)f->Hv;
  for (int q = 0; q < 3; q++) p.impl[q] = (const float *)f->impl[q];
  for (int q = 0; q < 2; q++) p.gsq[q] = (const float *)f->gsq[q];
  p.Fx = (const float *)f->F[0];
  p.Fy = (const float *)f->F[1];
  p.Fe = (const float *)f->F[2];
  p.wx = (const float *)f->wx;
  p.wy = (const float *)f->wy;
  int a = f->n0, b = 1 - f->n0;
  p.uh0 = f->uh[a]; p.ul0 = f->ul[a]; p.vh0 = f->vh[a]; p.vl0 = f->vl[a]; p.eh0 = f->eh[a]; p.el0 = f->el[a];
  p.uh1 = f->uh[b]; p.ul1 = f->ul[b]; p.vh1 = f->vh[b]; p.vl1 = f->vl[b]; p.eh1 = f->eh[b]; p.el1 = f->el[b];
  int s0 = f->g0, s1 = (f->g0 + 1) % 3, s2 = (f->g0 + 2) % 3;
  p.Gu1 = f->Gu[s0]; p.Gu2 = f->Gu[s1]; p.Gu3 = f->Gu[s2];
  p.Gv1 = f->Gv[s0]; p.Gv2 = f->Gv[s1]; p.Gv3 = f->Gv[s2];
  p.Ge1 = f->Ge[s0]; p.Ge2 = f->Ge[s1]; p.Ge3 = f->Ge[s2];
}

// the FP32 pair state: level and ring offsets, and the current level's arrays
void fused_indices(const swm_gpu_ctx *c, int *n0, int *g0) {
  *n0 = c->fused ? c->fused->n0 : 0;
  *g0 = c->fused ? c->fused->g0 : 0;
}
void fused_set_indices(swm_gpu_ctx *c, int n0, int g0) {
  c->fused->n0 = n0;
  c->fused->g0 = g0;
}
template <typename T>
__global__ void k_field_col0(const double *field, T *dst, int nx, int ny) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < ny) dst[j] = (T)field[(size_t)nx * j];
}

// after a time-dependent wind-stress stream's device record changed: the
// fused kernels read their own copy (row profile or field, in the path's
// precision), refreshed here from the stream's FP64 record
int fused_refresh_wind(swm_gpu_ctx *c, int id) {
  FusedState *f = c->fused;
  if (!f || !f->ready) return SWM_GPU_OK;
  const Stream &s = c->streams[id];
  if (s.is_const || s.type != SWM_FRC_WIND || c->cfg.mode != SWM_MODE_NONLINEAR) return SWM_GPU_OK;
  if (s.comp != SWM_CMP_ZONAL && s.comp != SWM_CMP_MERID) return SWM_GPU_OK;
  void *dst = s.comp == SWM_CMP_ZONAL ? f->wx : f->wy;
  if (!dst) return SWM_GPU_OK;
  if (f->wind_rows) {
    unsigned nb = (unsigned)((c->ny + 255) / 256);
    if (f->comp) k_field_col0<float><<<nb, 256, 0, c->stream>>>(s.d1, (float *)dst, c->nx, c->ny);
    else k_field_col0<double><<<nb, 256, 0, c->stream>>>(s.d1, (double *)dst, c->nx, c->ny);
  } else {
    unsigned nb = (unsigned)((c->n + 255) / 256);
    if (f->comp) k_to_f32<<<nb, 256, 0, c->stream>>>(s.d1, (float *)dst, c->n);
    else SWM_CK(cudaMemcpyAsync(dst, s.d1, c->n * 8, cudaMemcpyDeviceToDevice, c->stream));
  }
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

void fused_static(const swm_gpu_ctx *c, const float **He, const uint16_t **mask16, const float **Fe) {
  const FusedState *f = c->fused;
  *He = (const float *)f->He;
  *mask16 = f->mask16;
  *Fe = f->has_F ? (const float *)f->F[2] : nullptr;
}
const uint16_t *fused_mask_words(const swm_gpu_ctx *c) {
  return c->fused && !c->fused->m16h.empty() ? c->fused->m16h.data() : nullptr;
}
void fused_pair_level(const swm_gpu_ctx *c, const float *out[6]) {
  const FusedState *f = c->fused;
  int a = f->n0;
  out[0] = f->uh[a]; out[1] = f->ul[a]; out[2] = f->vh[a]; out[3] = f->vl[a]; out[4] = f->eh[a]; out[5] = f->el[a];
}

int monitor_march(swm_gpu_ctx *c, P32 &p, const MonitorStep &m);

// the step kernel's tiles (cut with S rows per warp now if the autotuner has
// not run: contexts the ensemble prepares)
static int march_grid(swm_gpu_ctx *c, const P32 &p, MarchGrid *g) {
  if (!c->march_tiles) FTRY(march_default_tiles(c, p, c->fused->m16h.data(), c->march_rows ? c->march_rows : 16));
  *g = MarchGrid{c->march_tiles, c->march_blocks};
  return SWM_GPU_OK;
}

// one step of the pair state; a monitored step (c->mon, taken here) runs the
// step kernel with its monitoring jobs
// ---- LINEARISED_MEAN_STATE on the fused paths ------------------------------
// The mean-state terms of the step -- the eta flux by the basic flow (with
// the reference's ip1(j) zonal index, Q3; swm_nonlinear_timestep_module.f90:
// 353-365), the relative vorticity times the basic flow (:385-388, :419-422),
// the basic-state vorticity part of the potential vorticity ((f + zeta_bs) /
// Dh, :230-257) and the basic-state part of the energy density (u U + v V,
// :259-310) -- are linear in the perturbation with static coefficients.  Two
// small kernels form them from the state the step reads and write F = Fc +
// terms into the forcing fields the fused kernels add, so the kernels keep
// the state-of-rest arithmetic (f / Dh, G eta).  FP64 arithmetic on either
// path; the FP32 pair state is read as hi + lo.
struct MSIn {
  const double *u, *v, *e;                              // FP64 state, or
  const float *uh, *ul, *vh, *vl, *eh, *el;             // the FP32 pair state
  __device__ __forceinline__ double U(size_t k) const { return u ? u[k] : (double)uh[k] + (double)ul[k]; }
  __device__ __forceinline__ double V(size_t k) const { return v ? v[k] : (double)vh[k] + (double)vl[k]; }
  __device__ __forceinline__ double E(size_t k) const { return e ? e[k] : (double)eh[k] + (double)el[k]; }
};

// relative vorticity at H points (vorticityFromVelocities2D, calc_lib.f90:
// 663-678) and u U + v V interpolated to eta points
__global__ void k_ms_diag(Dev d, MSIn s, const double *ubs, const double *vbs, double *zeta, double *ex) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const size_t k = i + (size_t)d.nx * j;
  const int im = i == 0 ? d.nx - 1 : i - 1, jm = j == 0 ? d.ny - 1 : j - 1;
  const int ip = i + 1 == d.nx ? 0 : i + 1, jp = j + 1 == d.ny ? 0 : j + 1;
  const size_t ki = im + (size_t)d.nx * j, kj = i + (size_t)d.nx * jm;
  const int8_t *oU = d.ocean[GU], *oV = d.ocean[GV];
  const double bcH = d.ocean[GH][k] == 1 ? 1. : d.lbc;
  const double *cH = d.cosl[GH], *cU = d.cosl[GU];
  const double dvdx = (oV[ki] + oV[k] == 0) ? 0. : bcH / (d.A * cH[j] * d.dLambda) * (s.V(k) - s.V(ki));
  const double dudy = (oU[k] + oU[kj] == 0) ? 0. : bcH * (cU[j] * s.U(k) - cU[jm] * s.U(kj)) / (d.A * d.dTheta);
  zeta[k] = dvdx - dudy / cH[j];
  const size_t kip = ip + (size_t)d.nx * j, kjp = i + (size_t)d.nx * jp;
  ex[k] = d.ocean[GE][k] == 1 ? (.5 * (s.U(kip) * ubs[kip]) + .5 * (s.U(k) * ubs[k])) +
                                   (.5 * (s.V(kjp) * vbs[kjp]) + .5 * (s.V(k) * vbs[k]))
                              : 0.;
}

template <typename T>
__global__ void k_ms_terms(Dev d, MSIn s, const double *ubs, const double *vbs, const double *zbs,
                           const double *zeta, const double *ex, const T *Fcx, const T *Fcy, const T *Fce, T *Fx,
                           T *Fy, T *Fe) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const int nx = d.nx, ny = d.ny;
  auto K = [nx](int a, int b) { return a + (size_t)nx * b; };
  const size_t k = K(i, j);
  const int im = i == 0 ? nx - 1 : i - 1, jm = j == 0 ? ny - 1 : j - 1;
  const int ip = i + 1 == nx ? 0 : i + 1, jp = j + 1 == ny ? 0 : j + 1;
  const int8_t *oE = d.ocean[GE], *oU = d.ocean[GU], *oV = d.ocean[GV];
  const double A = d.A, dL = d.dLambda, dT = d.dTheta;
  const double *cE = d.cosl[GE], *cU = d.cosl[GU], *cV = d.cosl[GV];
  const double *Dh = d.Hg[GH], *Du = d.Hg[GU], *Dv = d.Hg[GV];
  auto e2 = [&](size_t a, size_t b) {  // mask-normalised two-point mean of eta
    const double w = 1. / fmax((double)(oE[a] + oE[b]), 1.);
    return ((double)oE[a] * w) * s.E(a) + ((double)oE[b] * w) * s.E(b);
  };
  auto potx = [&](size_t a) { return zbs[a] / fmax(Dh[a], 2.220446049250313e-16); };
  double te = 0., tu = 0., tv = 0.;
  if (oE[k] == 1) {
    const int qi = j % nx == nx - 1 ? 0 : j % nx + 1;  // ip1(j) (Q3)
    const int qim = qi == 0 ? nx - 1 : qi - 1;
    const int jpm = jp == 0 ? ny - 1 : jp - 1;
    const double ea = e2(K(qi, j), K(qim, j)), eb = e2(k, K(im, j));
    const double ec = e2(K(i, jp), K(i, jpm)), ed = e2(k, K(i, jm));
    const double t = -(ea * ubs[K(ip, j)] - eb * ubs[k]) / dL - (cV[jp] * ec * vbs[K(i, jp)] - cV[j] * ed * vbs[k]) / dT;
    te = t / (A * cE[j]);
  }
  if (oU[k] == 1) {
    const size_t a1 = K(i, jp), a2 = K(im, j), a3 = K(im, jp);
    auto mv = [&](size_t a) { return oV[a] == 1 ? Dv[a] * s.V(a) : 0.; };
    tu = (.5 * zeta[a1] + .5 * zeta[k]) * (.25 * vbs[a1] + .25 * vbs[a2] + .25 * vbs[a3] + .25 * vbs[k]) +
         (.5 * potx(a1) + .5 * potx(k)) * (.25 * mv(a1) + .25 * mv(a2) + .25 * mv(a3) + .25 * mv(k)) -
         (ex[k] - ex[a2]) / (A * cU[j] * dL);
  }
  if (oV[k] == 1) {
    const size_t a1 = K(ip, j), a2 = K(i, jm), a4 = K(ip, jm);
    auto mu = [&](size_t a) { return oU[a] == 1 ? Du[a] * s.U(a) : 0.; };
    tv = -(.5 * zeta[a1] + .5 * zeta[k]) * (.25 * ubs[a1] + .25 * ubs[a2] + .25 * ubs[k] + .25 * ubs[a4]) -
         (.5 * potx(a1) + .5 * potx(k)) * (.25 * mu(a1) + .25 * mu(a2) + .25 * mu(k) + .25 * mu(a4)) -
         (ex[k] - ex[a2]) / (A * dT);
  }
  Fe[k] = (T)((double)Fce[k] + te);
  Fx[k] = (T)((double)Fcx[k] + tu);
  Fy[k] = (T)((double)Fcy[k] + tv);
}

// a time-dependent stream's part of the step's forcing, on the component's
// ocean points (swm_forcing_module.f90): oscillating (processOscillation
// :326-374) F += 2 (Re cos(omega t) - Im sin(omega t)); wind stress in the
// linear modes (processWindstress :274-324) F += scale d / (RHO0 [D]);
// custom and heating (:396-434, :539-552) F += d
template <typename T>
__global__ void k_stream_add(int n, int type, const double *d1, const double *d2, const int8_t *msk,
                             const double *D, double scale, double rho0, double r_iot, double i_iot, T *F) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (size_t)n) return;
  double a;
  if (type == SWM_FRC_OSC) {
    a = (2. * (d1[k] * r_iot - d2[k] * i_iot)) * msk[k];
  } else {
    if (msk[k] != 1) return;
    a = type == SWM_FRC_WIND ? scale * d1[k] / (D ? rho0 * D[k] : rho0) : d1[k];
  }
  F[k] = (T)((double)F[k] + a);
}

// a time-dependent eddy momentum flux stream's part of the step's forcing
// (the divergence of the flux on the u and v points, as the plain path's
// forcing update forms it: U2 into F_x, V2 into F_y, REY into both), in the
// same FP64 arithmetic, added to the fused paths' forcing fields
template <typename T>
__global__ void k_stream_emf(Dev d, int comp, const double *__restrict__ dd, T *Fx, T *Fy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = d.nx, ny = d.ny;
  if (i >= nx || j >= ny) return;
  auto ix = [nx](int ii, int jj) { return (size_t)ii + (size_t)nx * (size_t)jj; };
  auto p1 = [](int a, int n) { return a + 1 == n ? 0 : a + 1; };
  auto m1 = [](int a, int n) { return a == 0 ? n - 1 : a - 1; };
  const size_t k = ix(i, j);
  const double A = d.A;
  const double *He = d.Hg[GE], *Hu = d.Hg[GU], *Hv = d.Hg[GV], *H = d.Hg[GH];
  const double *cu = d.cosl[GU], *cv = d.cosl[GV];
  const int8_t *oU = d.ocean[GU], *oV = d.ocean[GV];
  // 4-point mean of dd from the H corners to the eta point (ii, jj)
  auto h2eta = [&](int ii, int jj) {
    return .25 * dd[ix(p1(ii, nx), p1(jj, ny))] + .25 * dd[ix(ii, jj)] + .25 * dd[ix(ii, p1(jj, ny))] +
           .25 * dd[ix(p1(ii, nx), jj)];
  };
  if (comp == SWM_CMP_U2) {
    if (oU[k] != 1) return;
    const int im = m1(i, nx);
    Fx[k] = (T)((double)Fx[k] +
                (-(h2eta(i, j) * He[k] - h2eta(im, j) * He[ix(im, j)]) / (2 * A * d.dLambda * cu[j] * Hu[k])));
  } else if (comp == SWM_CMP_V2) {
    if (oV[k] != 1) return;
    const int jm = m1(j, ny);
    Fy[k] = (T)((double)Fy[k] + (-(cu[j] * He[k] * h2eta(i, j) - cu[jm] * He[ix(i, jm)] * h2eta(i, jm)) /
                                  (8 * A * d.dTheta * cv[j] * Hv[k])));
  } else {
    const int jp = p1(j, ny), ip = p1(i, nx);
    if (oU[k] == 1)
      Fx[k] = (T)((double)Fx[k] + (-(cv[jp] * dd[ix(i, jp)] * H[ix(i, jp)] - cv[j] * dd[k] * H[k]) /
                                    (2 * A * d.dTheta * cu[j] * Hu[k])));
    if (oV[k] == 1)
      Fy[k] = (T)((double)Fy[k] +
                  (-(dd[ix(ip, j)] * H[ix(ip, j)] - dd[k] * H[k]) / (2 * A * d.dLambda * cv[j] * Hv[k])));
  }
}

// the mean-state terms of the coming step into the forcing fields
static int ms_terms(swm_gpu_ctx *c) {
  FusedState *f = c->fused;
  Dev d = c->dev();
  MSIn s = {};
  if (f->comp) {
    const int a = f->n0;
    s.uh = f->uh[a]; s.ul = f->ul[a]; s.vh = f->vh[a]; s.vl = f->vl[a]; s.eh = f->eh[a]; s.el = f->el[a];
  } else {
    s.u = d.u0; s.v = d.v0; s.e = d.eta0;
  }
  dim3 b(32, 8), g((c->nx + 31) / 32, (c->ny + 7) / 8);
  k_ms_diag<<<g, b, 0, c->stream>>>(d, s, c->ubs, c->vbs, f->ms_zeta, f->ms_ex);
  if (f->comp)
    k_ms_terms<float><<<g, b, 0, c->stream>>>(d, s, c->ubs, c->vbs, c->zbs, f->ms_zeta, f->ms_ex,
                                              (const float *)f->Fc[0], (const float *)f->Fc[1],
                                              (const float *)f->Fc[2], (float *)f->F[0], (float *)f->F[1],
                                              (float *)f->F[2]);
  else
    k_ms_terms<double><<<g, b, 0, c->stream>>>(d, s, c->ubs, c->vbs, c->zbs, f->ms_zeta, f->ms_ex,
                                               (const double *)f->Fc[0], (const double *)f->Fc[1],
                                               (const double *)f->Fc[2], (double *)f->F[0], (double *)f->F[1],
                                               (double *)f->F[2]);
  c->launches += 2;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// forcing of step itt: F = Fc (+ the mean-state terms) + the oscillating
// streams at the time the reference's forcing holds during step itt (set by
// the advance after step itt - 1: t = (itt - 1) dt)
static int dyn_forcing(swm_gpu_ctx *c, int64_t itt) {
  FusedState *f = c->fused;
  const size_t es = f->comp ? 4 : 8;
  if (f->lin_mean) FTRY(ms_terms(c));
  else
    for (int q = 0; q < 3; q++) SWM_CK(cudaMemcpyAsync(f->F[q], f->Fc[q], c->n * es, cudaMemcpyDeviceToDevice, c->stream));
  const double t = (double)(itt - 1) * c->cfg.dt;
  const int ns = (int)c->streams.size();
  std::vector<int> order;  // the reference's stream order: head, then reverse insertion
  if (ns > 0) order.push_back(0);
  for (int q = ns - 1; q >= 1; q--) order.push_back(q);
  const bool nonlin = c->cfg.mode == SWM_MODE_NONLINEAR;
  for (int q : order) {
    const Stream &st = c->streams[q];
    if (st.is_const) continue;
    if (st.type == SWM_FRC_WIND && nonlin) continue;  // recomputed by the step kernel
    if (st.type == SWM_FRC_EMF) {
      const Dev d = c->dev();
      const dim3 b(32, 8), g((c->nx + 31) / 32, (c->ny + 7) / 8);
      if (f->comp)
        k_stream_emf<float><<<g, b, 0, c->stream>>>(d, st.comp, st.d1, (float *)f->F[0], (float *)f->F[1]);
      else
        k_stream_emf<double><<<g, b, 0, c->stream>>>(d, st.comp, st.d1, (double *)f->F[0], (double *)f->F[1]);
      c->launches++;
      continue;
    }
    const int k = st.type == SWM_FRC_HEAT ? 2 : (st.comp == SWM_CMP_ZONAL ? 0 : (st.comp == SWM_CMP_MERID ? 1 : 2));
    const int g = k == 0 ? GU : (k == 1 ? GV : GE);
    const double *D = (st.type == SWM_FRC_WIND && c->cfg.barotropic) ? c->d_H[g] : nullptr;
    const double r = cos(st.omega * t), im = sin(st.omega * t);
    const unsigned nb = (unsigned)((c->n + 255) / 256);
    if (f->comp)
      k_stream_add<float><<<nb, 256, 0, c->stream>>>((int)c->n, st.type, st.d1, st.d2, c->d_ocean[g], D,
                                                     c->cfg.tau_scale, c->cfg.RHO0, r, im, (float *)f->F[k]);
    else
      k_stream_add<double><<<nb, 256, 0, c->stream>>>((int)c->n, st.type, st.d1, st.d2, c->d_ocean[g], D,
                                                      c->cfg.tau_scale, c->cfg.RHO0, r, im, (double *)f->F[k]);
    c->launches++;
  }
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

bool fused_dynamic_forcing(const swm_gpu_ctx *c) { return c->fused && c->fused->dyn_F; }

static int launch_fp32c(swm_gpu_ctx *c, int64_t itt) {
  P32 p;
  make_p32(c, itt, p);
  if (c->mon) {
    const MonitorStep *m = c->mon;
    c->mon = nullptr;
    return monitor_march(c, p, *m);
  }
  MarchGrid g;
  FTRY(march_grid(c, p, &g));
  march_launch(c, p, g);
  return SWM_GPU_OK;
}

int fused_step(swm_gpu_ctx *c, int64_t itt) {
  FTRY(fused_prepare(c));
  FusedState *f = c->fused;
  if (f->dyn_F) FTRY(dyn_forcing(c, itt));
  if (!f->comp) {
    FP<double> p;
    memset(&p, 0, sizeof(p));
    fill_common(c, p, itt);
    Dev d = c->dev();
    p.u0 = d.u0; p.v0 = d.v0; p.e0 = d.eta0;
    p.u1 = d.u1; p.v1 = d.v1; p.e1 = d.eta1;
    p.Gu1 = d.Gu[0]; p.Gu2 = d.Gu[1]; p.Gu3 = d.Gu[2];
    p.Gv1 = d.Gv[0]; p.Gv2 = d.Gv[1]; p.Gv3 = d.Gv[2];
    p.Ge1 = d.Ge[0]; p.Ge2 = d.Ge[1]; p.Ge3 = d.Ge[2];
    launch_fused<double>(c, p);
  } else {
    FTRY(launch_fp32c(c, itt));
    // the pair state advances here; the host-side advance only rotates the
    // FP64 level and ring indices
    f->n0 = 1 - f->n0;
    f->g0 = (f->g0 + 1) % 3;
  }
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

void fused_free(swm_gpu_ctx *c) {
  FusedState *f = c->fused;
  if (!f) return;
  auto F = [](void *p) { if (p) cudaFree(p); };
  for (int q = 0; q < 2; q++) { F(f->uh[q]); F(f->ul[q]); F(f->vh[q]); F(f->vl[q]); F(f->eh[q]); F(f->el[q]); }
  for (int q = 0; q < 3; q++) { F(f->Gu[q]); F(f->Gv[q]); F(f->Ge[q]); F(f->impl[q]); F(f->F[q]); }
  for (int q = 0; q < 2; q++) F(f->gsq[q]);
  F(f->mc); F(f->He); F(f->rows); F(f->Hu); F(f->Hv); F(f->wx); F(f->wy); F(f->rows32c); F(f->mask16);
  for (int q = 0; q < 3; q++) { F(f->dp[q]); F(f->Fc[q]); }
  F(f->ms_zeta); F(f->ms_ex);
  delete f;
  c->fused = nullptr;
}

}  // namespace swm

// ---------------------------------------------------------------------------
// Domain integrals (volume, potential and kinetic energy) in FP64
// ---------------------------------------------------------------------------
namespace swm {

// sum of the per-block partials, 3 x nb, by one block in a fixed order (the
// result does not depend on which block runs it)
__device__ __forceinline__ void integrals_final(const double *partial, int nb, double *out) {
  __shared__ double red[3][32];
  double a[3] = {0., 0., 0.};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int q = 0; q < 3; q++) a[q] += __ldcg(partial + (size_t)q * nb + b);
  for (int o = 16; o > 0; o >>= 1)
    for (int q = 0; q < 3; q++) a[q] += __shfl_down_sync(0xffffffffu, a[q], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 3; q++) red[q][warp] = a[q];
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[threadIdx.x][w];
    out[threadIdx.x] = t;
  }
}

constexpr int INTEGRALS_IL = 4;             // columns per thread in one row chunk
constexpr int INTEGRALS_MAX_THREADS = 512;  // threads per block
constexpr int INTEGRALS_MAX_BLOCKS = 1024;

// cell areas of one row: FP64, and as (hi, lo) binary32 pairs
struct RowAreas {
  const double *u, *v, *e;
  const float2 *pu, *pv, *pe;
};

// one thread's share of one (row, chunk) item: IL columns, their masks and
// the row's areas
struct IntChunk {
  int8_t mE[INTEGRALS_IL], mU[INTEGRALS_IL], mV[INTEGRALS_IL];
  double xe[INTEGRALS_IL], xu[INTEGRALS_IL], xv[INTEGRALS_IL];
  double du, dv, de;
};

// Domain sums of the FP64 state over ocean points.  The work is a row-major
// list of (row, chunk) items; a chunk is IL * blockDim.x columns, thread t
// holding columns t, t + blockDim.x, ...  Blocks stride through the list.  A
// thread issues all loads of an item (masks, values, areas; clamped in-row
// indices, no branch) before it adds any of them, so an item costs one
// memory round trip and the launch keeps a whole wave of items in flight.
// Per item a thread sums eta, eta^2, u^2, v^2 of its columns in FP64 and adds
// them times the row's cell area to its running totals.  Each block leaves
// its three sums in `partial`; the block that finishes last (counted in
// *done, which it resets to 0) adds the partials in block order into out[3].
// Every order is fixed by the launch shape: the result is deterministic.
__global__ void __launch_bounds__(INTEGRALS_MAX_THREADS)
    k_integrals(int nx, int ny, const int8_t *oU, const int8_t *oV, const int8_t *oE, RowAreas ar,
                const double *u, const double *v, const double *e, double G, double *partial, unsigned *done,
                double *out) {
  constexpr int IL = INTEGRALS_IL;
  __shared__ double red[4][INTEGRALS_MAX_THREADS / 32];
  __shared__ bool last;
  const int B = blockDim.x, W = IL * B;
  const int C = (nx + W - 1) / W;  // chunks per row
  const long long items = (long long)ny * C;
  auto load = [&](IntChunk &c, long long t) {
    const int j = (int)(t / C);
    const int i0 = (int)(t - (long long)j * C) * W + (int)threadIdx.x;
    const size_t row = (size_t)nx * j;
#pragma unroll
    for (int q = 0; q < IL; q++) {
      const int i = i0 + q * B;
      const bool in = i < nx;
      const size_t k = row + (in ? i : 0);
      c.mE[q] = in ? oE[k] : (int8_t)0;
      c.mU[q] = in ? oU[k] : (int8_t)0;
      c.mV[q] = in ? oV[k] : (int8_t)0;
      c.xe[q] = e[k];
      c.xu[q] = u[k];
      c.xv[q] = v[k];
    }
    c.du = ar.u[j];
    c.dv = ar.v[j];
    c.de = ar.e[j];
  };
  double s[4] = {0., 0., 0., 0.};
  for (long long t = blockIdx.x; t < items; t += gridDim.x) {
    IntChunk cur;
    load(cur, t);
    double r0 = 0., r1 = 0., ru = 0., rv = 0.;
#pragma unroll
    for (int q = 0; q < IL; q++) {
      const double ee = cur.mE[q] ? cur.xe[q] : 0.;
      const double uu = cur.mU[q] ? cur.xu[q] : 0.;
      const double vv = cur.mV[q] ? cur.xv[q] : 0.;
      r0 += ee;
      r1 += ee * ee;
      ru += uu * uu;
      rv += vv * vv;
    }
    s[0] += r0 * cur.de;
    s[1] += r1 * cur.de;
    s[2] += ru * cur.du;
    s[3] += rv * cur.dv;
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int q = 0; q < 4; q++) s[q] += __shfl_down_sync(0xffffffffu, s[q], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 4; q++) red[q][warp] = s[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double a[4] = {0., 0., 0., 0.};
    for (int w = 0; w < B / 32; w++)
      for (int q = 0; q < 4; q++) a[q] += red[q][w];
    partial[blockIdx.x] = a[0];
    partial[(size_t)gridDim.x + blockIdx.x] = 0.5 * G * a[1];
    partial[2 * (size_t)gridDim.x + blockIdx.x] = 0.5 * (a[2] + a[3]);
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  integrals_final(partial, gridDim.x, out);
  if (threadIdx.x == 0) *done = 0u;
}

// Domain sums of the pair state, marching as the step kernel does: warp
// task t covers columns 32 s .. 32 s + 31 (s = t % strips, lane = column) and
// rows IP_ROWS g .. IP_ROWS g + IP_ROWS - 1 (g = t / strips).  Each row's
// values, packed mask word and cell areas are loaded one row ahead into
// registers; each lane adds its ocean points times the row's areas into
// (hi, lo) pair sums (the monitored step kernel's arithmetic).  The warps of
// a block are added in order in FP64, and the blocks as in k_integrals: the
// last block to finish adds their partials in block order into out[3] and
// resets *done.  Fixed order throughout.
#ifndef IP_ROWS_N
#define IP_ROWS_N 16
#endif
constexpr int IP_ROWS = IP_ROWS_N;  // rows of one warp task
constexpr int IP_WARPS = 8;         // warps per block

__global__ void __launch_bounds__(32 * IP_WARPS)
    k_integrals_pair(int nx, int ny, const uint16_t *__restrict__ m16, RowAreas ar, const float *__restrict__ uh,
                     const float *__restrict__ ul, const float *__restrict__ vh, const float *__restrict__ vl,
                     const float *__restrict__ eh, const float *__restrict__ el, double G, double *partial,
                     unsigned *done, double *out) {
  __shared__ double red[4][IP_WARPS];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int strips = (nx + 31) / 32, groups = (ny + IP_ROWS - 1) / IP_ROWS;
  const long long tasks = (long long)strips * groups;
  F2 acc[4];
  for (long long t = (long long)blockIdx.x * IP_WARPS + warp; t < tasks; t += (long long)gridDim.x * IP_WARPS) {
    const int st = (int)(t % strips), g = (int)(t / strips);
    const int i = 32 * st + lane;
    const bool col = i < nx;
    const int ic = col ? i : nx - 1;
    const int j0 = g * IP_ROWS, j1 = min(j0 + IP_ROWS, ny);
    unsigned nm;
    float nuh, nul, nvh, nvl, neh, nel;
    float2 npu, npv, npe;
    auto load = [&](int j) {
      const size_t k = (size_t)nx * j + ic;
      nm = col ? m16[k] : 0u;
      nuh = uh[k]; nul = ul[k]; nvh = vh[k]; nvl = vl[k]; neh = eh[k]; nel = el[k];
      npu = ar.pu[j]; npv = ar.pv[j]; npe = ar.pe[j];
    };
    load(j0);
    for (int j = j0; j < j1; j++) {
      const unsigned m = nm;
      const float xuh = nuh, xul = nul, xvh = nvh, xvl = nvl, xeh = neh, xel = nel;
      const float2 apu = npu, apv = npv, ape = npe;
      if (j + 1 < j1) load(j + 1);
      F2 sq;
      if ((m >> 3) & 1u) {
        F2 x;
        x.h = xeh;
        x.l = xel;
        acc[0].add_prod(ape, x);
        sq_pair(xeh, xel, sq.h, sq.l);
        acc[1].add_prod(ape, sq);
      }
      if ((m >> 1) & 1u) {
        sq_pair(xuh, xul, sq.h, sq.l);
        acc[2].add_prod(apu, sq);
      }
      if ((m >> 2) & 1u) {
        sq_pair(xvh, xvl, sq.h, sq.l);
        acc[3].add_prod(apv, sq);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float h = __shfl_down_sync(0xffffffffu, acc[q].h, o), l = __shfl_down_sync(0xffffffffu, acc[q].l, o);
      acc[q].add(h, l);
    }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 4; q++) red[q][warp] = acc[q].value();
  __syncthreads();
  if (threadIdx.x == 0) {
    double a[4] = {0., 0., 0., 0.};
    for (int w = 0; w < IP_WARPS; w++)
      for (int q = 0; q < 4; q++) a[q] += red[q][w];
    partial[blockIdx.x] = a[0];
    partial[(size_t)gridDim.x + blockIdx.x] = 0.5 * G * a[1];
    partial[2 * (size_t)gridDim.x + blockIdx.x] = 0.5 * (a[2] + a[3]);
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  integrals_final(partial, gridDim.x, out);
  if (threadIdx.x == 0) *done = 0u;
}

// blocks of k_integrals_pair: a block per IP_WARPS tasks, at most
// INTEGRALS_MAX_BLOCKS (the warps then take several tasks each)
static int integrals_pair_blocks(int nx, int ny) {
  const long long tasks = (long long)((nx + 31) / 32) * ((ny + IP_ROWS - 1) / IP_ROWS);
  return (int)std::max(1LL, std::min<long long>((tasks + IP_WARPS - 1) / IP_WARPS, INTEGRALS_MAX_BLOCKS));
}

// launch shape of k_integrals for an nx x ny grid: the fewest threads (a
// multiple of 32, at most INTEGRALS_MAX_THREADS) that cover a row in equal
// chunks of IL columns each, and one wave of blocks (at most one per item)
static int integrals_shape_fp64(int nx, int ny, int *threads, int *blocks) {
  const int need = (nx + INTEGRALS_IL - 1) / INTEGRALS_IL;
  const int chunks = (need + INTEGRALS_MAX_THREADS - 1) / INTEGRALS_MAX_THREADS;
  const int thr = std::min(INTEGRALS_MAX_THREADS, ((need + chunks - 1) / chunks + 31) / 32 * 32);
  const int W = INTEGRALS_IL * thr;
  const long long items = (long long)ny * ((nx + W - 1) / W);
  int dev = 0, sms = 0, per_sm = 0;
  SWM_CK(cudaGetDevice(&dev));
  SWM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SWM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrals, thr, 0));
  const long long wave = (long long)std::max(per_sm, 1) * std::max(sms, 1);
  *threads = thr;
  *blocks = (int)std::max(1LL, std::min(items, std::min<long long>(wave, INTEGRALS_MAX_BLOCKS)));
  return SWM_GPU_OK;
}

// the state k_integrals reads (pair state of the fused paths once it is
// ready, else the FP64 state) and its cached launch shape
struct IntegralsInput {
  bool comp;
  const void *u, *v, *e;
  const float *ul, *vl, *el;
};

static IntegralsInput integrals_input(swm_gpu_ctx *c) {
  FusedState *f = c->fused;
  if (f && f->ready && f->comp) {
    const int a = f->n0;
    return {true, f->uh[a], f->vh[a], f->eh[a], f->ul[a], f->vl[a], f->el[a]};
  }
  return {false, c->u[c->n0], c->v[c->n0], c->eta[c->n0], nullptr, nullptr, nullptr};
}

static int integrals_run(swm_gpu_ctx *c, const RowAreas &ar, double *partial, unsigned *done, double *out) {
  const IntegralsInput in = integrals_input(c);
  int *sh = c->integrals_shape;  // {tuned, threads, blocks} of k_integrals
  if (!in.comp && sh[0] != 0) {
    const int rc = integrals_shape_fp64(c->nx, c->ny, &sh[1], &sh[2]);
    if (rc != SWM_GPU_OK) return rc;
    sh[0] = 0;
  }
  const int8_t *oU = c->d_ocean[GU], *oV = c->d_ocean[GV], *oE = c->d_ocean[GE];
  if (in.comp)
    k_integrals_pair<<<integrals_pair_blocks(c->nx, c->ny), 32 * IP_WARPS, 0, c->stream>>>(
        c->nx, c->ny, c->fused->mask16, ar, (const float *)in.u, in.ul, (const float *)in.v, in.vl,
        (const float *)in.e, in.el, c->cfg.G, partial, done, out);
  else
    k_integrals<<<sh[2], sh[1], 0, c->stream>>>(c->nx, c->ny, oU, oV, oE, ar, (const double *)in.u,
                                                 (const double *)in.v, (const double *)in.e, c->cfg.G, partial,
                                                 done, out);
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// (hi, lo) binary32 split of an FP64 area, the same on the host and the device
__host__ __device__ inline float2 area_pair(double a) {
  const float h = (float)a;
  return make_float2(h, (float)(a - (double)h));
}

__global__ void k_expand_rows(const double *rows, double *field, int nx, int ny) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < (size_t)nx * ny) field[k] = rows[k / nx];
}

// the wind rows in binary32; waits for the previous kernel on the stream
// (which may read dst) when launched as its programmatic dependent
__global__ void k_rows_f32(const double *rows, float *dst, int ny) {
  grid_dep_wait();
  grid_dep_trigger();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < ny) dst[j] = (float)rows[j];
}

}  // namespace swm

// scratch of swm_gpu_integrals, owned by its context (allocated on the first
// call, freed with the context)
struct IntegralScratch {
  double *area = nullptr;     // FP64 cell areas of the u, v, eta rows, 3 x Ny
  float2 *pairs = nullptr;    // the same as (hi, lo) binary32 pairs, 3 x Ny
  double *partial = nullptr;  // 3 x INTEGRALS_MAX_BLOCKS
  double *out = nullptr;      // 3
  unsigned *done = nullptr;   // blocks finished in the running reduction (0 between calls)
  double *host = nullptr;     // pinned
  double *mpartial = nullptr;  // per-block sums of monitored steps, two steps' worth
  size_t mpartial_n = 0;
  float *w_alt = nullptr;      // alternate wind rows of monitored steps (Ny)
  double *res = nullptr;       // results of monitored steps for unmapped host arrays
  size_t res_n = 0;
};

namespace swm {
void integrals_free(swm_gpu_ctx *c) {
  IntegralScratch *S = c->integrals;
  if (!S) return;
  cudaFree(S->area);
  cudaFree(S->pairs);
  cudaFree(S->partial);
  cudaFree(S->out);
  cudaFree(S->done);
  cudaFree(S->mpartial);
  cudaFree(S->w_alt);
  cudaFree(S->res);
  cudaFreeHost(S->host);
  delete S;
  c->integrals = nullptr;
}
}  // namespace swm

extern "C" {

int swm_gpu_set_stream_rows(swm_gpu_ctx *c, int id, const double *r1, const double *r2) {
  SWM_ON_DEVICE(c ? c->device : -1);
  return swm::stream_rows(c, id, r1, r2, nullptr);
}

}  // extern "C"

namespace swm {
// rows r1 (and r2) of stream id into the stream's device record, or into the
// fused path's row copy.  d1: r1 as the device may read it in place (r1 in
// host-mapped pinned memory), or null; it is used where the rows go through
// one small conversion kernel, which then reads the host array directly
// instead of a staged copy.
int stream_rows(swm_gpu_ctx *c, int id, const double *r1, const double *r2, const double *d1) {
  SWM_REQUIRE(c && id >= 0 && id < (int)c->streams.size() && r1, "swm_gpu_set_stream_rows: bad arguments");
  const Stream &s = c->streams[id];
  FusedState *f = c->fused;
  bool fused_rows = f && f->ready && f->wind_rows && !s.is_const && s.type == SWM_FRC_WIND;
  if (fused_rows && f->comp && d1) {
    float *dst = (float *)(s.comp == SWM_CMP_ZONAL ? f->wx : f->wy);
    SWM_CK(launch_programmatic(k_rows_f32, dim3((c->ny + 255) / 256), dim3(256), c->stream, d1, dst, c->ny));
    c->launches++;
    SWM_CK(cudaGetLastError());
    return SWM_GPU_OK;
  }
  if (!c->rows_buf) SWM_CK(cudaMalloc((void **)&c->rows_buf, 2 * (size_t)c->ny * 8));
  double *d_rows = c->rows_buf;
  SWM_CK(cudaMemcpyAsync(d_rows, r1, c->ny * 8, cudaMemcpyHostToDevice, c->stream));
  if (r2) SWM_CK(cudaMemcpyAsync(d_rows + c->ny, r2, c->ny * 8, cudaMemcpyHostToDevice, c->stream));
  if (fused_rows) {
    void *dst = s.comp == SWM_CMP_ZONAL ? f->wx : f->wy;
    if (f->comp) {
      k_rows_f32<<<(c->ny + 255) / 256, 256, 0, c->stream>>>(d_rows, (float *)dst, c->ny);
    } else {
      SWM_CK(cudaMemcpyAsync(dst, d_rows, c->ny * 8, cudaMemcpyDeviceToDevice, c->stream));
    }
  } else {
    unsigned nb = (unsigned)((c->n + 255) / 256);
    k_expand_rows<<<nb, 256, 0, c->stream>>>(d_rows, s.d1, c->nx, c->ny);
    if (r2) k_expand_rows<<<nb, 256, 0, c->stream>>>(d_rows + c->ny, s.d2, c->nx, c->ny);
  }
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

}  // namespace swm

// the context's integrals scratch (allocated on the first call)
static int integrals_scratch(swm_gpu_ctx *c, IntegralScratch **out) {
  IntegralScratch *S = c->integrals;
  const size_t ny = (size_t)c->ny;
  if (!S) {
    S = c->integrals = new IntegralScratch();
    const HostGrid &g = c->hg;
    std::vector<double> area(3 * ny);
    std::vector<float2> pairs(3 * ny);
    const double A = c->cfg.A;
    const int grids[3] = {GU, GV, GE};
    for (int q = 0; q < 3; q++)
      for (size_t j = 0; j < ny; j++) {
        area[q * ny + j] = A * A * g.cosl[grids[q]][j] * g.dLambda * g.dTheta;
        pairs[q * ny + j] = area_pair(area[q * ny + j]);
      }
    SWM_CK(cudaMalloc((void **)&S->area, 3 * ny * sizeof(double)));
    SWM_CK(cudaMalloc((void **)&S->pairs, 3 * ny * sizeof(float2)));
    SWM_CK(cudaMalloc((void **)&S->partial, 3 * (size_t)INTEGRALS_MAX_BLOCKS * sizeof(double)));
    SWM_CK(cudaMalloc((void **)&S->out, 3 * sizeof(double)));
    SWM_CK(cudaMalloc((void **)&S->done, sizeof(unsigned)));
    SWM_CK(cudaMemset(S->done, 0, sizeof(unsigned)));
    SWM_CK(cudaMallocHost((void **)&S->host, 3 * sizeof(double)));
    SWM_CK(cudaMemcpy(S->area, area.data(), 3 * ny * sizeof(double), cudaMemcpyHostToDevice));
    SWM_CK(cudaMemcpy(S->pairs, pairs.data(), 3 * ny * sizeof(float2), cudaMemcpyHostToDevice));
  }
  *out = S;
  return SWM_GPU_OK;
}

// the three sums of the current state into the context's device scratch S->out
static int integrals_launch(swm_gpu_ctx *c) {
  IntegralScratch *S = nullptr;
  FTRY(integrals_scratch(c, &S));
  const size_t ny = (size_t)c->ny;
  const RowAreas ar{S->area, S->area + ny, S->area + 2 * ny, S->pairs, S->pairs + ny, S->pairs + 2 * ny};
  return integrals_run(c, ar, S->partial, S->done, S->out);
}

namespace swm {
// the integrals of the current state into dst[3] (device or host-mapped
// memory; null: the context's device result slot); *where gets the address
// written
int integrals_to(swm_gpu_ctx *c, double *dst, double **where) {
  IntegralScratch *S = nullptr;
  FTRY(integrals_scratch(c, &S));
  const size_t ny = (size_t)c->ny;
  if (!dst) dst = S->out;
  if (where) *where = dst;
  const RowAreas ar{S->area, S->area + ny, S->area + 2 * ny, S->pairs, S->pairs + ny, S->pairs + 2 * ny};
  return integrals_run(c, ar, S->partial, S->done, dst);
}

// ---- swm_gpu_run_monitor on the FP32 pair path ----------------------------

bool monitor_fast(const swm_gpu_ctx *c) {
  const FusedState *f = c->fused;
  return c->cfg.path == SWM_PATH_FUSED_FP32C && f && f->ready && f->comp && !c->cfg.frozen_flow && !f->dyn_F;
}

bool monitor_rows_fast(const swm_gpu_ctx *c, int sid) {
  const FusedState *f = c->fused;
  if (!monitor_fast(c) || sid < 0 || sid >= (int)c->streams.size() || !f->wind_rows) return false;
  const Stream &s = c->streams[sid];
  return !s.is_const && s.type == SWM_FRC_WIND && (s.comp == SWM_CMP_ZONAL ? f->wx : f->wy) != nullptr;
}

static int grow(double **p, size_t *have, size_t need) {
  if (*have >= need) return SWM_GPU_OK;
  if (*p) SWM_CK(cudaFree(*p));
  *p = nullptr;
  *have = 0;
  SWM_CK(cudaMalloc((void **)p, need * sizeof(double)));
  *have = need;
  return SWM_GPU_OK;
}

int fused_monitor_inputs(swm_gpu_ctx *c, int comp, float **wind_rows, const float2 **area_pairs) {
  const FusedState *f = c->fused;
  SWM_REQUIRE(f && f->ready && f->comp, "monitored ensemble steps: member has no FP32 pair state");
  IntegralScratch *S = nullptr;
  FTRY(integrals_scratch(c, &S));
  *area_pairs = S->pairs;
  *wind_rows = nullptr;
  if (f->wind_rows) *wind_rows = (float *)(comp == SWM_CMP_ZONAL ? (f->wind_x ? f->wx : nullptr)
                                                                 : (f->wind_y ? f->wy : nullptr));
  return SWM_GPU_OK;
}

int monitor_buffers(swm_gpu_ctx *c, int64_t nsteps, int sid, bool rows, bool res, MonitorBufs *b) {
  IntegralScratch *S = nullptr;
  FTRY(integrals_scratch(c, &S));
  const FusedState *f = c->fused;
  P32 p;
  make_p32(c, 3, p);
  MarchGrid g;
  FTRY(march_grid(c, p, &g));
  b->nb = g.blocks;
  FTRY(grow(&S->mpartial, &S->mpartial_n, 2 * 4 * (size_t)b->nb));
  b->partial[0] = S->mpartial;
  b->partial[1] = S->mpartial + 4 * (size_t)b->nb;
  b->w[0] = b->w[1] = nullptr;
  b->w_merid = 0;
  if (rows) {
    if (!S->w_alt) SWM_CK(cudaMalloc((void **)&S->w_alt, (size_t)c->ny * sizeof(float)));
    b->w_merid = c->streams[sid].comp != SWM_CMP_ZONAL;
    b->w[0] = (float *)(b->w_merid ? f->wy : f->wx);
    b->w[1] = S->w_alt;
  }
  b->res = nullptr;
  if (res) {
    FTRY(grow(&S->res, &S->res_n, 3 * (size_t)nsteps));
    b->res = S->res;
  }
  return SWM_GPU_OK;
}

// the first monitored step's wind rows, converted before its step kernel
int monitor_rows_first(swm_gpu_ctx *c, const double *rows_dev, float *w) {
  SWM_CK(launch_programmatic(k_rows_f32, dim3((c->ny + 255) / 256), dim3(256), c->stream, rows_dev, w, c->ny));
  c->launches++;
  return SWM_GPU_OK;
}

// the step kernel of a monitored step
int monitor_march(swm_gpu_ctx *c, P32 &p, const MonitorStep &m) {
  IntegralScratch *S = nullptr;
  FTRY(integrals_scratch(c, &S));
  if (m.w_now) (m.w_merid ? p.wy : p.wx) = m.w_now;
  const MarchInteg mi{S->pairs, m.partial, m.prev_partial, m.prev_out, m.next_rows, m.next_w, c->cfg.G, c->ny, 1};
  MarchGrid g;
  FTRY(march_grid(c, p, &g));
  march_launch(c, p, g, &mi);
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// the last monitored step's integrals
int monitor_finish(swm_gpu_ctx *c, const MonitorBufs &b, const double *partial, double *out) {
  march_integrals_final(partial, b.nb, c->cfg.G, out, c->stream);
  c->launches++;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// after a monitored run whose last step read the alternate rows: the fused
// state's own rows take them, so later steps see the last rows set
int monitor_keep_rows(swm_gpu_ctx *c, const MonitorBufs &b, int last) {
  if (b.w[0] && last == 1)
    SWM_CK(cudaMemcpyAsync(b.w[0], b.w[1], (size_t)c->ny * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  return SWM_GPU_OK;
}
}  // namespace swm

extern "C" {

int swm_gpu_integrals(swm_gpu_ctx *c, double *out3) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5 && out3, "swm_gpu_integrals: bad arguments");
  FTRY(integrals_launch(c));
  IntegralScratch *S = c->integrals;
  SWM_CK(cudaMemcpyAsync(S->host, S->out, 3 * 8, cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  for (int q = 0; q < 3; q++) out3[q] = S->host[q];
  return SWM_GPU_OK;
}

int swm_gpu_integrals_async(swm_gpu_ctx *c, double *out3, int64_t *ticket) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5 && out3 && ticket, "swm_gpu_integrals_async: bad arguments");
  FTRY(integrals_launch(c));
  SWM_CK(cudaMemcpyAsync(out3, c->integrals->out, 3 * 8, cudaMemcpyDeviceToHost, c->stream));
  return async_record(c, ticket);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Domain integrals without any allocation
//
// The same reduction as swm_gpu_integrals (same kernels, block count and cell
// areas, so the same sums bit for bit), but every intermediate lives in one
// fixed array compiled into this library.  It is meant for callers that must
// not allocate in the middle of a time loop: a host whose device memory is
// already reserved in full by its own pool (a cudaMalloc there fails or makes
// the pool give memory back), and a host that runs other streams concurrently
// (cudaFree and the first cudaMallocHost can synchronise the whole device and
// so stall them).  Limits: grids of at most SWM_NOALLOC_MAX_NY rows; one
// scratch array per device, so two calls that overlap in time on one device
// (from two threads, or two contexts) race on it and must be serialised by
// the caller.
// ---------------------------------------------------------------------------
namespace swm {

constexpr size_t NOALLOC_MAX_NY = SWM_NOALLOC_MAX_NY;
// area[3 * MAX_NY] | pairs[3 * MAX_NY] (float2, one double slot each) |
// partial[3 * INTEGRALS_MAX_BLOCKS] | out[3] | block counter (one 8-byte slot,
// zero at load, left at zero by every call): 418 KB per device
constexpr size_t NOALLOC_DOUBLES = 6 * NOALLOC_MAX_NY + 3 * (size_t)INTEGRALS_MAX_BLOCKS + 4;
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];
// device address of the scratch per device ordinal, looked up on first use
constexpr int NOALLOC_MAX_DEVICES = 64;
static std::atomic<double *> g_noalloc_ptr[NOALLOC_MAX_DEVICES];

// cell areas per row, A^2 cos(lat) dLambda dTheta, for the u, v and eta rows,
// the product in the order swm_gpu_integrals forms it on the host, and their
// binary32 pairs
__global__ void k_area_rows(const double *cos_u, const double *cos_v, const double *cos_e, double A, double dL,
                            double dT, int ny, double *area, float2 *pairs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ny) return;
  const double *cs[3] = {cos_u, cos_v, cos_e};
  for (int q = 0; q < 3; q++) {
    const double a = A * A * cs[q][j] * dL * dT;
    area[(size_t)q * ny + j] = a;
    pairs[(size_t)q * ny + j] = area_pair(a);
  }
}

}  // namespace swm

extern "C" int swm_gpu_integrals_noalloc(swm_gpu_ctx *c, double *out3) {
  SWM_ON_DEVICE(c ? c->device : -1);
  using namespace swm;
  SWM_REQUIRE(c && c->stage >= 5 && out3, "swm_gpu_integrals_noalloc: bad arguments");
  if (c->ny > SWM_NOALLOC_MAX_NY) {
    set_error("swm_gpu_integrals_noalloc: the grid has " + std::to_string(c->ny) +
              " rows; the fixed scratch serves at most " + std::to_string(SWM_NOALLOC_MAX_NY));
    return SWM_GPU_EINVAL;
  }
  // the call ends by waiting for its result, which a stream under capture
  // cannot do (the wait would invalidate the capture)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  SWM_CK(cudaStreamIsCapturing(c->stream, &cap));
  SWM_REQUIRE(cap == cudaStreamCaptureStatusNone,
              "swm_gpu_integrals_noalloc: the context's stream is being captured; this call waits for its result");
  int dev = -1;
  SWM_CK(cudaGetDevice(&dev));
  SWM_REQUIRE(dev >= 0 && dev < NOALLOC_MAX_DEVICES, "swm_gpu_integrals_noalloc: device ordinal out of range");
  // set-up, once per device: the address of this device's copy of the array
  double *scr = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!scr) {
    SWM_CK(cudaGetSymbolAddress((void **)&scr, g_noalloc_scratch));
    g_noalloc_ptr[dev].store(scr, std::memory_order_release);
  }
  // every slot below but the counter is written before it is read; the
  // counter starts at zero with the module and each reduction resets it
  const size_t ny = (size_t)c->ny;
  double *area = scr;
  float2 *pairs = reinterpret_cast<float2 *>(scr + 3 * NOALLOC_MAX_NY);
  double *partial = scr + 6 * NOALLOC_MAX_NY, *out = partial + 3 * (size_t)INTEGRALS_MAX_BLOCKS;
  unsigned *done = reinterpret_cast<unsigned *>(out + 3);
  const HostGrid &g = c->hg;
  k_area_rows<<<(c->ny + 127) / 128, 128, 0, c->stream>>>(c->d_cos[GU], c->d_cos[GV], c->d_cos[GE], c->cfg.A,
                                                          g.dLambda, g.dTheta, c->ny, area, pairs);
  c->launches++;
  SWM_CK(cudaGetLastError());
  const RowAreas ar{area, area + ny, area + 2 * ny, pairs, pairs + ny, pairs + 2 * ny};
  FTRY(integrals_run(c, ar, partial, done, out));
  SWM_CK(cudaMemcpyAsync(out3, out, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}
