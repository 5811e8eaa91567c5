// api.cu -- the extern "C" entry points of include/swm_gpu.h.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include "ctx.h"
#include "fused32.h"

namespace swm {
static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
}  // namespace swm

using namespace swm;

swm::Dev swm_gpu_ctx::dev() const {
  Dev d;
  memset(&d, 0, sizeof(d));
  d.nx = nx;
  d.ny = ny;
  d.mode = cfg.mode;
  d.qbf = cfg.quadratic_friction;
  d.barotropic = cfg.barotropic;
  d.lateral_mixing = cfg.lateral_mixing;
  d.dt = cfg.dt;
  d.G = cfg.G;
  d.A = cfg.A;
  d.dLambda = hg.dLambda;
  d.dTheta = hg.dTheta;
  d.minD = cfg.minD;
  d.tau_scale = cfg.tau_scale;
  d.RHO0 = cfg.RHO0;
  d.lbc = cfg.lbc;
  d.pdiv = pdiv ? 1 : 0;
  d.r_dLambda = 1. / hg.dLambda;
  d.r_dTheta = 1. / hg.dTheta;
  d.AdT = cfg.A * hg.dTheta;
  d.r_AdT = 1. / d.AdT;
  d.prow = prow;
  for (int q = 0; q < 3; q++) d.rimpl[q] = rimpl[q];
  for (int q = 0; q < 4; q++) {
    d.ocean[q] = d_ocean[q];
    d.cosl[q] = d_cos[q];
    d.tanl[q] = d_tan[q];
    d.f[q] = d_f[q];
    d.Hg[q] = d_H[q];
  }
  d.u0 = u[n0];
  d.v0 = v[n0];
  d.eta0 = eta[n0];
  d.u1 = u[1 - n0];
  d.v1 = v[1 - n0];
  d.eta1 = eta[1 - n0];
  for (int s = 0; s < 3; s++) {
    d.Gu[s] = Gu[(g0 + s) % 3];
    d.Gv[s] = Gv[(g0 + s) % 3];
    d.Ge[s] = Ge[(g0 + s) % 3];
  }
  if (cfg.mode == SWM_MODE_NONLINEAR) {
    d.D = Dbuf[0];
    d.Dh = Dbuf[1];
    d.Du = Dbuf[2];
    d.Dv = Dbuf[3];
  } else {  // swm_vars.f90:100-105: the thickness arrays are the grid depths
    d.D = d_H[GE];
    d.Dh = d_H[GH];
    d.Du = d_H[GU];
    d.Dv = d_H[GV];
  }
  d.edens = edens;
  d.pot = pot;
  d.zeta = zeta;
  d.mu = mu;
  d.mv = mv;
  d.pll = pll;
  d.plt = plt;
  d.lmu = lmu;
  d.lmv = lmv;
  d.impl_u = impl[0];
  d.impl_v = impl[1];
  d.impl_e = impl[2];
  d.gsq_u = gsq[0];
  d.gsq_v = gsq[1];
  d.Fx = F[0];
  d.Fy = F[1];
  d.Fe = F[2];
  d.Fxc = Fc[0];
  d.Fyc = Fc[1];
  d.Fec = Fc[2];
  d.ubs = ubs;
  d.vbs = vbs;
  d.zbs = zbs;
  return d;
}

// allocations are zeroed on the context's stream, so that later kernels on
// that (non-blocking) stream are ordered after the zeroing
static cudaStream_t g_alloc_stream = nullptr;
static int dalloc(double **p, size_t n) {
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(double));
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return SWM_GPU_ENOMEM;
  }
  e = cudaMemsetAsync(*p, 0, n * sizeof(double), g_alloc_stream);
  if (e != cudaSuccess) {
    set_error(std::string("cudaMemset: ") + cudaGetErrorString(e));
    return SWM_GPU_ECUDA;
  }
  return SWM_GPU_OK;
}

#define TRY(x)                  \
  do {                          \
    int rc_ = (x);              \
    if (rc_ != SWM_GPU_OK) return rc_; \
  } while (0)

static int h2d(swm_gpu_ctx *c, double *dst, const double *src, size_t count) {
  SWM_CK(cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return SWM_GPU_OK;
}
static int d2h(swm_gpu_ctx *c, double *dst, const double *src, size_t count) {
  SWM_CK(cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}

static void invalidate_graph(swm_gpu_ctx *c) {
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
}

extern "C" {

const char *swm_gpu_last_error(void) { return g_last_error.c_str(); }

int swm_gpu_create(const swm_gpu_config *cfg, swm_gpu_ctx **out) {
  SWM_REQUIRE(cfg && out, "swm_gpu_create: null argument");
  SWM_REQUIRE(cfg->nx >= 3 && cfg->ny >= 3, "swm_gpu_create: Nx and Ny must be >= 3");
  SWM_REQUIRE(cfg->dt > 0, "swm_gpu_create: dt must be positive");
  SWM_REQUIRE(cfg->mode >= 0 && cfg->mode <= 3, "swm_gpu_create: unknown mode");
  SWM_REQUIRE(cfg->path >= 0 && cfg->path <= 2, "swm_gpu_create: unknown path");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("swm_gpu_create: no CUDA device is visible");
    return SWM_GPU_ECUDA;
  }
  swm_gpu_ctx *c = new swm_gpu_ctx();
  c->cfg = *cfg;
  if (cudaGetDevice(&c->device) != cudaSuccess) c->device = -1;
  c->nx = cfg->nx;
  c->ny = cfg->ny;
  c->n = (size_t)cfg->nx * cfg->ny;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    delete c;
    return SWM_GPU_ECUDA;
  }
  *out = c;
  return SWM_GPU_OK;
}

int swm_gpu_destroy(swm_gpu_ctx *c) {
  SWM_ON_DEVICE(c ? c->device : -1);
  if (!c) return SWM_GPU_OK;
  cudaStreamSynchronize(c->stream);
  invalidate_graph(c);
  fused_free(c);
  sor_free(c);
  integrals_free(c);
  trc32_free(c);
  diag_free(c);
  auto F = [](void *p) { if (p) cudaFree(p); };
  for (int q = 0; q < 4; q++) {
    F(c->d_ocean[q]); F(c->d_cos[q]); F(c->d_tan[q]); F(c->d_f[q]); F(c->d_lat[q]); F(c->d_H[q]);
    F(c->Dbuf[q]); F(c->bh[q]);
  }
  for (int q = 0; q < 2; q++) { F(c->u[q]); F(c->v[q]); F(c->eta[q]); F(c->gsq[q]); }
  for (int q = 0; q < 3; q++) { F(c->Gu[q]); F(c->Gv[q]); F(c->Ge[q]); F(c->impl[q]); F(c->glin[q]); F(c->F[q]); F(c->Fc[q]); }
  F(c->edens); F(c->pot); F(c->zeta); F(c->mu); F(c->mv); F(c->pll); F(c->plt); F(c->lmu); F(c->lmv);
  F(c->ones); F(c->latp[0]); F(c->latp[1]); F(c->latuv); F(c->prow); F(c->rimpl[0]); F(c->rimpl[1]);
  F(c->rimpl[2]); F(c->pdiv_bad); F(c->ubs); F(c->vbs); F(c->zbs); F(c->trc_coeff); F(c->rows_buf); F(c->march_tiles);
  for (auto &s : c->streams) { F(s.d1); F(s.d2); F(s.rec[0]); F(s.rec[1]); }
  for (auto &t : c->tracers) {
    F(t.CH[0]); F(t.CH[1]); F(t.G[0]); F(t.G[1]); F(t.G[2]); F(t.C); F(t.C0); F(t.gamma); F(t.impl);
    F(t.uhc); F(t.vhc); F(t.diff);
  }
  for (auto e : c->async_ev) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
  return SWM_GPU_OK;
}

int swm_gpu_synchronize(swm_gpu_ctx *c) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c, "null context");
  SWM_CK(cudaStreamSynchronize(c->stream));
  return march_ring_check();
}

void *swm_gpu_stream(swm_gpu_ctx *c) { return c ? (void *)c->stream : nullptr; }
int64_t swm_gpu_launch_count(swm_gpu_ctx *c) {
  SWM_ON_DEVICE(c ? c->device : -1); return c ? c->launches : -1; }

int swm_gpu_step_shape(swm_gpu_ctx *c, double *rows, double *masked_cost, int *blocks) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && rows && masked_cost && blocks, "swm_gpu_step_shape: bad arguments");
  *rows = c->march_tiles ? c->march_S : 0.;
  *masked_cost = c->march_tiles ? c->march_slow : 0.;
  *blocks = c->march_tiles ? c->march_blocks : 0;
  return SWM_GPU_OK;
}

int swm_gpu_domain(swm_gpu_ctx *c, const double *H, const int8_t *Hmiss) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage == 0, "swm_gpu_domain: call once, first");
  TRY(host_domain(c, H, Hmiss));
  g_alloc_stream = c->stream;
  size_t n = c->n;
  int ny = c->ny;
  const HostGrid &g = c->hg;
  for (int q = 0; q < 4; q++) {
    SWM_CK(cudaMalloc((void **)&c->d_ocean[q], n));
    SWM_CK(cudaMemcpy(c->d_ocean[q], g.ocean[q].data(), n, cudaMemcpyHostToDevice));
    TRY(dalloc(&c->d_cos[q], ny));
    TRY(dalloc(&c->d_tan[q], ny));
    TRY(dalloc(&c->d_f[q], ny));
    TRY(dalloc(&c->d_lat[q], ny));
    TRY(dalloc(&c->d_H[q], n));
    SWM_CK(cudaMemcpy(c->d_cos[q], g.cosl[q].data(), ny * 8, cudaMemcpyHostToDevice));
    SWM_CK(cudaMemcpy(c->d_tan[q], g.tanl[q].data(), ny * 8, cudaMemcpyHostToDevice));
    SWM_CK(cudaMemcpy(c->d_f[q], g.f[q].data(), ny * 8, cudaMemcpyHostToDevice));
    SWM_CK(cudaMemcpy(c->d_lat[q], g.lat[q].data(), ny * 8, cudaMemcpyHostToDevice));
    SWM_CK(cudaMemcpy(c->d_H[q], g.H[q].data(), n * 8, cudaMemcpyHostToDevice));
  }
  for (int q = 0; q < 2; q++) {
    TRY(dalloc(&c->u[q], n)); TRY(dalloc(&c->v[q], n)); TRY(dalloc(&c->eta[q], n));
  }
  for (int q = 0; q < 3; q++) {
    TRY(dalloc(&c->Gu[q], n)); TRY(dalloc(&c->Gv[q], n)); TRY(dalloc(&c->Ge[q], n));
    TRY(dalloc(&c->impl[q], n)); TRY(dalloc(&c->glin[q], n)); TRY(dalloc(&c->F[q], n)); TRY(dalloc(&c->Fc[q], n));
  }
  for (int q = 0; q < 2; q++) TRY(dalloc(&c->gsq[q], n));
  TRY(dalloc(&c->edens, n)); TRY(dalloc(&c->pot, n)); TRY(dalloc(&c->zeta, n));
  TRY(dalloc(&c->mu, n)); TRY(dalloc(&c->mv, n));
  TRY(dalloc(&c->pll, n)); TRY(dalloc(&c->plt, n)); TRY(dalloc(&c->lmu, n)); TRY(dalloc(&c->lmv, n));
  TRY(dalloc(&c->ubs, n)); TRY(dalloc(&c->vbs, n)); TRY(dalloc(&c->zbs, n));
  if (c->cfg.mode == SWM_MODE_NONLINEAR) {
    for (int q = 0; q < 4; q++) { TRY(dalloc(&c->Dbuf[q], n)); TRY(plain_fill(c, c->Dbuf[q], 1.)); }
  }
  if (c->cfg.lateral_mixing && c->cfg.mixing_kind == SWM_MIX_BIHARMONIC) {
    for (int q = 0; q < 4; q++) TRY(dalloc(&c->bh[q], n));
    TRY(dalloc(&c->ones, n));
    TRY(plain_fill(c, c->ones, 1.));
  }
  for (int q = 0; q < 3; q++) TRY(plain_fill(c, c->impl[q], 1.));
  c->n0 = 0;
  c->g0 = 0;
  c->stage = 1;
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}

// SWM_timestep_init: basic state, then computeD/RelVort/PotVort/EDens/
// MassFluxes at itt = 0 (which overwrites the grid depths in linear modes).
int swm_gpu_timestep_init(swm_gpu_ctx *c, const double *psi_bs) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage == 1, "swm_gpu_timestep_init: call after swm_gpu_domain");
  if (c->cfg.mode == SWM_MODE_LIN_MEAN) {
    SWM_REQUIRE(psi_bs, "swm_gpu_timestep_init: LINEARISED_MEAN_STATE needs psi_bs");
    host_basic_state(c, psi_bs);
    TRY(h2d(c, c->ubs, c->hg.ubs.data(), c->n));
    TRY(h2d(c, c->vbs, c->hg.vbs.data(), c->n));
    TRY(h2d(c, c->zbs, c->hg.zbs.data(), c->n));
  }
  TRY(plain_diagnostics(c, 0));
  for (int q = 0; q < 4; q++) TRY(d2h(c, c->hg.H[q].data(), c->d_H[q], c->n));
  c->stage = 2;
  return SWM_GPU_OK;
}

int swm_gpu_add_damping(swm_gpu_ctx *c, int term, int type, double value, double sl_length,
                        double sl_cutoff, int loc, const double *file_data) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage == 2, "swm_gpu_add_damping: call after swm_gpu_timestep_init");
  SWM_REQUIRE(term >= 0 && term <= 4, "swm_gpu_add_damping: unknown term");
  SWM_REQUIRE(type >= 0 && type <= 2, "swm_gpu_add_damping: unknown type");
  SWM_REQUIRE(type != SWM_DAMP_FILE || file_data, "swm_gpu_add_damping: file type needs data");
  SWM_REQUIRE(type != SWM_DAMP_SPONGE || sl_length > 0, "swm_gpu_add_damping: sponge length must be > 0");
  host_damping_add(c, term, type, value, sl_length, sl_cutoff, loc, file_data);
  return SWM_GPU_OK;
}

int swm_gpu_finish_damping(swm_gpu_ctx *c) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage == 2, "swm_gpu_finish_damping: call after swm_gpu_timestep_init");
  host_damping_finish(c);
  const HostGrid &g = c->hg;
  for (int q = 0; q < 3; q++) {
    TRY(h2d(c, c->impl[q], g.impl[q].data(), c->n));
    TRY(h2d(c, c->glin[q], g.glin[q].data(), c->n));
  }
  for (int q = 0; q < 2; q++) TRY(h2d(c, c->gsq[q], g.gsq[q].data(), c->n));
  SWM_CK(cudaStreamSynchronize(c->stream));
  c->stage = 3;
  return SWM_GPU_OK;
}

int swm_gpu_add_stream(swm_gpu_ctx *c, int type, int comp, double omega, int is_const, const double *d1,
                       const double *d2, int *id) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage == 3, "swm_gpu_add_stream: call after swm_gpu_finish_damping");
  SWM_REQUIRE(type >= 0 && type <= 4, "swm_gpu_add_stream: unknown forcing type");
  SWM_REQUIRE(c->streams.size() < 64, "swm_gpu_add_stream: too many streams");
  Stream s;
  s.type = type;
  s.comp = comp;
  s.omega = omega;
  // SWM_forcing_initStream :627-638
  if (type == SWM_FRC_OSC) s.is_const = 0;
  else if (type == SWM_FRC_WIND && c->cfg.mode == SWM_MODE_NONLINEAR) s.is_const = 0;
  else s.is_const = is_const ? 1 : 0;
  g_alloc_stream = c->stream;
  TRY(dalloc(&s.d1, c->n));
  TRY(dalloc(&s.d2, c->n));
  if (d1) TRY(h2d(c, s.d1, d1, c->n));
  if (d2) TRY(h2d(c, s.d2, d2, c->n));
  c->streams.push_back(s);
  if (id) *id = (int)c->streams.size() - 1;
  return SWM_GPU_OK;
}

int swm_gpu_set_stream_data(swm_gpu_ctx *c, int id, const double *d1, const double *d2) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && id >= 0 && id < (int)c->streams.size(), "swm_gpu_set_stream_data: bad stream id");
  if (d1) TRY(h2d(c, c->streams[id].d1, d1, c->n));
  if (d2) TRY(h2d(c, c->streams[id].d2, d2, c->n));
  if (d1) TRY(fused_refresh_wind(c, id));
  return SWM_GPU_OK;
}

int swm_gpu_stream_records(swm_gpu_ctx *c, int id, int part, int nrec, const double *records) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && id >= 0 && id < (int)c->streams.size() && (part == 1 || part == 2) && nrec > 0 && records,
              "swm_gpu_stream_records: bad arguments");
  Stream &s = c->streams[id];
  double *&r = s.rec[part - 1];
  if (r) cudaFree(r);
  r = nullptr;
  SWM_CK(cudaMalloc((void **)&r, (size_t)nrec * c->n * 8));
  s.nrec[part - 1] = nrec;
  SWM_CK(cudaMemcpyAsync(r, records, (size_t)nrec * c->n * 8, cudaMemcpyHostToDevice, c->stream));
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}

int swm_gpu_stream_interp(swm_gpu_ctx *c, int id, int part, int r0, int r1, double t, double t0, double t1) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && id >= 0 && id < (int)c->streams.size() && (part == 1 || part == 2),
              "swm_gpu_stream_interp: bad arguments");
  Stream &s = c->streams[id];
  const int nr = s.nrec[part - 1];
  SWM_REQUIRE(s.rec[part - 1] && r0 >= 0 && r0 < nr && r1 < nr, "swm_gpu_stream_interp: records not set or bad index");
  TRY(stream_interp(c, s.rec[part - 1], part == 1 ? s.d1 : s.d2, r0, r1, t, t0, t1));
  if (part == 1) TRY(fused_refresh_wind(c, id));
  return SWM_GPU_OK;
}

int swm_gpu_forcing_init(swm_gpu_ctx *c) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage == 3, "swm_gpu_forcing_init: call after swm_gpu_finish_damping");
  TRY(plain_forcing_update(c, 0, 1));
  TRY(plain_forcing_update(c, 0, 0));
  c->stage = 4;
  return SWM_GPU_OK;
}

static int swm_advance_impl(swm_gpu_ctx *c, int64_t itt);

int swm_gpu_initial_conditions(swm_gpu_ctx *c, const double *eta, const double *u, const double *v) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage == 4, "swm_gpu_initial_conditions: call after swm_gpu_forcing_init");
  size_t n = c->n;
  std::vector<double> buf(n);
  const HostGrid &g = c->hg;
  const double *src[3] = {eta, u, v};
  double **dst[3] = {c->eta, c->u, c->v};
  const int grids[3] = {GE, GU, GV};
  for (int f = 0; f < 3; f++) {
    for (size_t k = 0; k < n; k++) buf[k] = src[f] ? g.ocean[grids[f]][k] * src[f][k] : 0.;
    TRY(h2d(c, dst[f][1 - c->n0], buf.data(), n));
    SWM_CK(cudaMemsetAsync(dst[f][c->n0], 0, n * 8, c->stream));
  }
  SWM_CK(cudaStreamSynchronize(c->stream));
  TRY(swm_advance_impl(c, 0));
  c->stage = 5;
  return SWM_GPU_OK;
}

static int swm_step_impl(swm_gpu_ctx *c, int64_t itt) {
  // FP32 tracers read the level the SWM step reads, so they go first
  if (trc32_active(c)) TRY(trc32_step(c, itt));
  if (c->cfg.frozen_flow) {  // prescribed flow: only the tracers step
    if (!c->tracers.empty() && !trc32_active(c)) TRY(tracer_step(c, itt));
    return SWM_GPU_OK;
  }
  if (c->cfg.path == SWM_PATH_PLAIN_FP64) TRY(plain_step(c, itt));
  else TRY(fused_step(c, itt));
  if (!c->tracers.empty() && !trc32_active(c)) TRY(tracer_step(c, itt));
  return SWM_GPU_OK;
}

// SWM_advance: level swap, increment ring rotation, diagnostics, forcing
// (fused paths keep their diagnostics and wind forcing inside the step
// kernel; the FP64 diagnostic arrays are refreshed on demand, or every step
// when tracers read them)
static int swm_advance_impl(swm_gpu_ctx *c, int64_t itt) {
  c->advances++;
  const bool t32 = trc32_active(c), t64 = !c->tracers.empty() && !t32;
  if (c->cfg.frozen_flow && itt > 0) {  // state, diagnostics and forcing stay
    if (t32) trc32_advance(c);
    if (t64) TRY(tracer_advance(c));
    return SWM_GPU_OK;
  }
  c->n0 = 1 - c->n0;
  c->g0 = (c->g0 + 1) % 3;
  bool plain = c->cfg.path == SWM_PATH_PLAIN_FP64 || itt == 0;
  if (!plain && t64) TRY(fused_sync_state(c));
  if (plain || t64) {
    TRY(plain_diagnostics(c, itt));
    TRY(plain_forcing_update(c, itt, 0));
  }
  if (itt > 0) {
    if (t32) trc32_advance(c);
    if (t64) TRY(tracer_advance(c));
  }
  return SWM_GPU_OK;
}

int swm_gpu_step(swm_gpu_ctx *c, int64_t itt) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5, "swm_gpu_step: model not initialised");
  SWM_REQUIRE(itt >= 1, "swm_gpu_step: itt starts at 1");
  return swm_step_impl(c, itt);
}

int swm_gpu_advance(swm_gpu_ctx *c, int64_t itt) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5, "swm_gpu_advance: model not initialised");
  return swm_advance_impl(c, itt);
}

// From itt = 3 on the Adams-Bashforth weights are fixed, and without tracers
// or oscillating forcing no kernel argument depends on itt; the pointers
// cycle with the two time levels and the three increment slots, so a block of
// six steps is captured once and replayed as a CUDA graph.
constexpr int GRAPH_STEPS = 6;

static bool graph_eligible(const swm_gpu_ctx *c) {
  if (!c->tracers.empty() && !trc32_active(c)) return false;
  for (const Stream &s : c->streams)
    if (s.type == SWM_FRC_OSC) return false;
  return true;
}

// records steps itt0+1 .. itt0+GRAPH_STEPS without running them; the host
// indices go round the full cycle and end where they started
static int graph_capture(swm_gpu_ctx *c, int64_t itt0) {
  invalidate_graph(c);
  if (c->cfg.path != SWM_PATH_PLAIN_FP64) TRY(fused_prepare(c));  // allocates on first use
  else TRY(plain_prepare(c));
  const int n0 = c->n0, g0 = c->g0, phase = (int)(c->advances % GRAPH_STEPS);
  const int64_t l0 = c->launches;
  SWM_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc = SWM_GPU_OK;
  for (int s = 1; s <= GRAPH_STEPS && rc == SWM_GPU_OK; s++) {
    rc = swm_step_impl(c, itt0 + s);
    if (rc == SWM_GPU_OK) rc = swm_advance_impl(c, itt0 + s);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  const int64_t nl = c->launches - l0;
  c->launches = l0;
  if (rc != SWM_GPU_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc != SWM_GPU_OK) return rc;
    set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    return SWM_GPU_ECUDA;
  }
  SWM_REQUIRE(c->n0 == n0 && c->g0 == g0, "swm_gpu_run: index cycle is not a multiple of the graph length");
  e = cudaGraphInstantiate(&c->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    c->graph = nullptr;
    set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return SWM_GPU_ECUDA;
  }
  c->graph_launches = nl;
  c->graph_phase = phase;
  return SWM_GPU_OK;
}

int swm_gpu_run(swm_gpu_ctx *c, int64_t itt0, int64_t nsteps) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5, "swm_gpu_run: model not initialised");
  const bool graphs = graph_eligible(c) && nsteps >= 2 * GRAPH_STEPS;
  int64_t s = 1;
  while (s <= nsteps) {
    const int64_t itt = itt0 + s;
    if (graphs && itt >= 3 && nsteps - s + 1 >= GRAPH_STEPS) {
      if (!c->graph) TRY(graph_capture(c, itt - 1));
      if (c->advances % GRAPH_STEPS == c->graph_phase) {
        SWM_CK(cudaGraphLaunch(c->graph, c->stream));
        c->launches += c->graph_launches;
        s += GRAPH_STEPS;
        continue;
      }
    }
    TRY(swm_step_impl(c, itt));
    TRY(swm_advance_impl(c, itt));
    s++;
  }
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

// device address of a host array the device may read and write in place
// (pinned, mapped into the device's address space), else null
static double *mapped_view(const double *h) {
  if (!h) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost && a.devicePointer ? (double *)a.devicePointer : nullptr;
}

// A monitored run issued from C with no host wait per step: for each step,
// the step's wind-stress row profile goes up, the step and advance run, and
// the domain integrals of the new state come down into out3 + 3 s; one wait
// at the end.
//
// On the FP32 pair path each step is one kernel launch: the step kernel sums
// the state it writes per block, and its extra block 0 converts the next
// step's rows (read in place from pinned host memory, into the other half of
// a double buffer) and finishes the previous step's integrals, written in
// place into pinned host memory.  Other paths, and arrays that are not
// pinned, take the general route: staged rows, the reduction kernel after the
// advance, and copies.
int swm_gpu_run_monitor(swm_gpu_ctx *c, int64_t itt0, int64_t nsteps, int stream_id, const double *rows1,
                        const double *rows2, double *out3) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5 && nsteps > 0 && out3, "swm_gpu_run_monitor: bad arguments");
  SWM_REQUIRE(!rows1 || (stream_id >= 0 && stream_id < (int)c->streams.size()),
              "swm_gpu_run_monitor: bad stream id");
  const size_t ny = (size_t)c->ny;
  const double *rows_dev = mapped_view(rows1);
  double *out_dev = mapped_view(out3);
  auto set_rows = [&](int64_t s) -> int {
    if (!rows1) return SWM_GPU_OK;
    return stream_rows(c, stream_id, rows1 + s * ny, rows2 ? rows2 + s * ny : nullptr,
                       rows_dev ? rows_dev + s * ny : nullptr);
  };
  int64_t s = 0;
  // the general route, until the pair path is ready (its first step prepares it)
  for (; s < nsteps && !monitor_fast(c); s++) {
    const int64_t itt = itt0 + s + 1;
    TRY(set_rows(s));
    TRY(swm_step_impl(c, itt));
    TRY(swm_advance_impl(c, itt));
    double *where = nullptr;
    TRY(integrals_to(c, out_dev ? out_dev + 3 * s : nullptr, &where));
    if (!out_dev) SWM_CK(cudaMemcpyAsync(out3 + 3 * s, where, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  if (s < nsteps) {
    const int64_t s0 = s;
    const bool rows_job = rows1 && rows_dev && monitor_rows_fast(c, stream_id);
    MonitorBufs b;
    TRY(monitor_buffers(c, nsteps, stream_id, rows_job, !out_dev, &b));
    double *res = out_dev ? out_dev : b.res;  // step s's integrals at res + 3 s
    if (rows_job) TRY(monitor_rows_first(c, rows_dev + s0 * ny, b.w[0]));
    for (; s < nsteps; s++) {
      const int64_t k = s - s0, itt = itt0 + s + 1;
      MonitorStep m = {};
      if (rows_job) {
        m.w_now = b.w[k & 1];
        m.w_merid = b.w_merid;
        if (s + 1 < nsteps) {
          m.next_rows = rows_dev + (s + 1) * ny;
          m.next_w = b.w[(k + 1) & 1];
        }
      } else {
        TRY(set_rows(s));
      }
      m.partial = b.partial[k & 1];
      if (k > 0) {
        m.prev_partial = b.partial[(k - 1) & 1];
        m.prev_out = res + 3 * (s - 1);
      }
      c->mon = &m;
      const int rc = swm_step_impl(c, itt);
      const bool taken = c->mon == nullptr;
      c->mon = nullptr;
      TRY(rc);
      SWM_REQUIRE(taken, "swm_gpu_run_monitor: the step did not run the monitored step kernel");
      TRY(swm_advance_impl(c, itt));
    }
    const int last = (int)((nsteps - 1 - s0) & 1);
    TRY(monitor_finish(c, b, b.partial[last], res + 3 * (nsteps - 1)));
    if (rows_job) TRY(monitor_keep_rows(c, b, last));
    if (!out_dev)
      SWM_CK(cudaMemcpyAsync(out3 + 3 * s0, b.res + 3 * s0, 3 * sizeof(double) * (size_t)(nsteps - s0),
                             cudaMemcpyDeviceToHost, c->stream));
  }
  SWM_CK(cudaStreamSynchronize(c->stream));
  return SWM_GPU_OK;
}

static const double *field_ptr(swm_gpu_ctx *c, int f, double **wptr) {
  Dev d = c->dev();
  double *p = nullptr;
  switch (f) {
    case SWM_F_U: p = d.u0; break;
    case SWM_F_V: p = d.v0; break;
    case SWM_F_ETA: p = d.eta0; break;
    case SWM_F_D: p = d.D; break;
    case SWM_F_DH: p = d.Dh; break;
    case SWM_F_DU: p = d.Du; break;
    case SWM_F_DV: p = d.Dv; break;
    case SWM_F_EDENS: p = d.edens; break;
    case SWM_F_POT: p = d.pot; break;
    case SWM_F_ZETA: p = d.zeta; break;
    case SWM_F_MU: p = d.mu; break;
    case SWM_F_MV: p = d.mv; break;
    case SWM_F_H: p = c->d_H[GH]; break;
    case SWM_F_HU: p = c->d_H[GU]; break;
    case SWM_F_HV: p = c->d_H[GV]; break;
    case SWM_F_HETA: p = c->d_H[GE]; break;
    case SWM_F_IMPL_U: p = c->impl[0]; break;
    case SWM_F_IMPL_V: p = c->impl[1]; break;
    case SWM_F_IMPL_ETA: p = c->impl[2]; break;
    case SWM_F_GAMMA_LIN_U: p = c->glin[0]; break;
    case SWM_F_GAMMA_LIN_V: p = c->glin[1]; break;
    case SWM_F_GAMMA_LIN_ETA: p = c->glin[2]; break;
    case SWM_F_GAMMA_SQ_U: p = c->gsq[0]; break;
    case SWM_F_GAMMA_SQ_V: p = c->gsq[1]; break;
    case SWM_F_FX: p = d.Fx; break;
    case SWM_F_FY: p = d.Fy; break;
    case SWM_F_FETA: p = d.Fe; break;
    case SWM_F_U_BS: p = d.ubs; break;
    case SWM_F_V_BS: p = d.vbs; break;
    case SWM_F_ZETA_BS: p = d.zbs; break;
    case SWM_F_LATMIX_U: p = d.lmu; break;
    case SWM_F_LATMIX_V: p = d.lmv; break;
    case SWM_F_GU: p = c->Gu[(c->g0 + 1) % 3]; break;  // newest increment after advance = slot 2
    case SWM_F_GV: p = c->Gv[(c->g0 + 1) % 3]; break;
    case SWM_F_GETA: p = c->Ge[(c->g0 + 1) % 3]; break;
    default: p = nullptr;
  }
  if (wptr) *wptr = p;
  return p;
}

// device copy of a field as of the current state (fused paths: the FP64
// state and the diagnostics are formed from the FP32 pair state first)
static int field_device(swm_gpu_ctx *c, int f, const double **out) {
  if (c->cfg.path != SWM_PATH_PLAIN_FP64 && c->stage >= 5 && c->fused) {
    TRY(fused_sync_state(c));
    if (f >= SWM_F_D && f <= SWM_F_MV) TRY(plain_diagnostics(c, 1));
    if (f >= SWM_F_FX && f <= SWM_F_FETA) TRY(plain_forcing_update(c, 1, 0));
  }
  if (f == SWM_F_PSI) {
    SWM_REQUIRE(c->stage >= 5, "streamfunction: model not initialised");
    TRY(device_streamfunction(c));
    *out = c->psi;
    return SWM_GPU_OK;
  }
  const double *p = field_ptr(c, f, nullptr);
  SWM_REQUIRE(p, "unknown field or not allocated");
  *out = p;
  return SWM_GPU_OK;
}

int swm_gpu_get_field(swm_gpu_ctx *c, int f, double *out) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 1 && out, "swm_gpu_get_field: bad arguments");
  const double *p = nullptr;
  TRY(field_device(c, f, &p));
  return d2h(c, out, p, c->n);
}

}  // extern "C"

constexpr int ASYNC_RING = 64;

// marks the work queued so far on the context's stream with a new ticket
int swm::async_record(swm_gpu_ctx *c, int64_t *ticket) {
  if (c->async_ev.empty()) {
    c->async_ev.resize(ASYNC_RING);
    for (auto &e : c->async_ev) SWM_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  const int64_t t = c->async_next++;
  SWM_CK(cudaEventRecord(c->async_ev[t % ASYNC_RING], c->stream));
  *ticket = t;
  return SWM_GPU_OK;
}

extern "C" {

int swm_gpu_get_field_async(swm_gpu_ctx *c, int f, double *out, int64_t *ticket) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 1 && out && ticket, "swm_gpu_get_field_async: bad arguments");
  const double *p = nullptr;
  TRY(field_device(c, f, &p));
  SWM_CK(cudaMemcpyAsync(out, p, c->n * 8, cudaMemcpyDeviceToHost, c->stream));
  return async_record(c, ticket);
}

int swm_gpu_wait(swm_gpu_ctx *c, int64_t ticket) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && ticket >= 0 && ticket < c->async_next, "swm_gpu_wait: unknown ticket");
  SWM_CK(cudaEventSynchronize(c->async_ev[ticket % ASYNC_RING]));
  return SWM_GPU_OK;
}

int swm_gpu_ready(swm_gpu_ctx *c, int64_t ticket) {
  SWM_ON_DEVICE(c ? c->device : -1);
  if (!c || ticket < 0 || ticket >= c->async_next) return -1;
  cudaError_t e = cudaEventQuery(c->async_ev[ticket % ASYNC_RING]);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  set_error(std::string("swm_gpu_ready: ") + cudaGetErrorString(e));
  return -1;
}

int swm_gpu_host_register(void *host, int64_t bytes) {
  SWM_REQUIRE(host && bytes > 0, "swm_gpu_host_register: bad arguments");
  SWM_CK(cudaHostRegister(host, (size_t)bytes, cudaHostRegisterDefault));
  return SWM_GPU_OK;
}

int swm_gpu_host_unregister(void *host) {
  SWM_REQUIRE(host, "swm_gpu_host_unregister: bad arguments");
  SWM_CK(cudaHostUnregister(host));
  return SWM_GPU_OK;
}

int swm_gpu_diag_accumulate(swm_gpu_ctx *c, int slot, int f, int square, double weight) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5 && slot >= 0 && slot < 4096, "swm_gpu_diag_accumulate: bad arguments");
  const double *p = nullptr;
  TRY(field_device(c, f, &p));
  return diag_accumulate(c, slot, p, square, weight);
}

int swm_gpu_diag_mean(swm_gpu_ctx *c, int slot, double *out, double *count) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && out, "swm_gpu_diag_mean: bad arguments");
  if (!c->psi_tmp) {  // the zonal-sum scratch doubles as the staging buffer
    SWM_CK(cudaMalloc((void **)&c->psi, c->n * 8));
    SWM_CK(cudaMalloc((void **)&c->psi_tmp, c->n * 8));
  }
  TRY(diag_mean(c, slot, c->psi_tmp, count));
  return d2h(c, out, c->psi_tmp, c->n);
}

int swm_gpu_set_field(swm_gpu_ctx *c, int f, const double *in) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 1 && in, "swm_gpu_set_field: bad arguments");
  double *p = nullptr;
  field_ptr(c, f, &p);
  SWM_REQUIRE(p, "swm_gpu_set_field: unknown field or not allocated");
  // static fields (depths, damping, drag, constant forcing, basic state)
  // that the fused paths copied when they set up their own state
  const bool static_field = (f >= SWM_F_H && f <= SWM_F_FETA) || (f >= SWM_F_U_BS && f <= SWM_F_ZETA_BS);
  SWM_REQUIRE(!(static_field && c->cfg.path != SWM_PATH_PLAIN_FP64 && c->fused),
              "swm_gpu_set_field: on the fused paths, set static fields before the first step");
  TRY(h2d(c, p, in, c->n));
  SWM_CK(cudaStreamSynchronize(c->stream));
  if (c->cfg.path != SWM_PATH_PLAIN_FP64 && c->stage >= 5 && f <= SWM_F_ETA) TRY(fused_load_state(c));
  if (f == SWM_F_IMPL_U || f == SWM_F_IMPL_V || f == SWM_F_IMPL_ETA) {
    c->pdiv_ready = false;  // the plain path's reciprocals of the damping factors are formed again
    invalidate_graph(c);
  }
  return SWM_GPU_OK;
}

int swm_gpu_get_metric(swm_gpu_ctx *c, int which, int grid, double *out) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 1 && out && which >= 0 && which <= 3 && grid >= 0 && grid <= 3,
              "swm_gpu_get_metric: bad arguments");
  const HostGrid &g = c->hg;
  const std::vector<double> *src[4] = {&g.lat[grid], &g.cosl[grid], &g.tanl[grid], &g.f[grid]};
  memcpy(out, src[which]->data(), sizeof(double) * c->ny);
  return SWM_GPU_OK;
}

int swm_gpu_get_mask(swm_gpu_ctx *c, int grid, int8_t *out) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 1 && out && grid >= 0 && grid <= 3, "swm_gpu_get_mask: bad arguments");
  memcpy(out, c->hg.ocean[grid].data(), c->n);
  return SWM_GPU_OK;
}

int swm_gpu_streamfunction(swm_gpu_ctx *c, double *psi) {
  SWM_ON_DEVICE(c ? c->device : -1);
  SWM_REQUIRE(c && c->stage >= 5 && psi, "swm_gpu_streamfunction: bad arguments");
  return swm_gpu_get_field(c, SWM_F_PSI, psi);
}

}  // extern "C"
