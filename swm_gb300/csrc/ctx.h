// ctx.h -- internal state of one SWM model instance on the GPU.
//
// Device layout: every 2-D field is an unpadded Fortran-order (Nx, Ny) array
// (row j holds i = 0..Nx-1 contiguously), so host <-> device copies need no
// transpose.  Time levels and the Adams-Bashforth increment history are
// rotated by index, never copied (the reference copies N0p1 -> N0 and shifts
// G(:,:,1:2) = G(:,:,2:3) every step: swm_module.f90:91-113,
// swm_nonlinear_timestep_module.f90:134-148).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include <string>
#include <vector>
#include "../../include/swm_gpu.h"

namespace swm {

struct MonitorStep;

enum { GH = 0, GU = 1, GV = 2, GE = 3 };  // grid ids: H (corner), u, v, eta

void set_error(const std::string &msg);

#define SWM_CK(call)                                                              \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      ::swm::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));        \
      return SWM_GPU_ECUDA;                                                       \
    }                                                                             \
  } while (0)

// Every entry point runs on the device its context was created on: the guard
// makes that device current for the call and restores the caller's device
// when it returns (nothing happens when it is already current).
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    int cur = -1;
    if (dev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard &) = delete;
  DeviceGuard &operator=(const DeviceGuard &) = delete;
};
#define SWM_ON_DEVICE(dev) ::swm::DeviceGuard swm_device_guard_(dev)

#define SWM_REQUIRE(cond, msg)                                                    \
  do {                                                                            \
    if (!(cond)) {                                                                \
      ::swm::set_error(msg);                                                      \
      return SWM_GPU_EINVAL;                                                      \
    }                                                                             \
  } while (0)

// Host copy of the grid as domain_module/grid_module build it.
struct HostGrid {
  int nx = 0, ny = 0;
  double dLambda = 0, dTheta = 0, D2R = 0;
  std::vector<double> lat[4], lon[4], cosl[4], tanl[4], sinl[4], f[4];
  std::vector<int8_t> ocean[4];
  std::vector<double> H[4];     // H, H_u, H_v, H_eta (grid%H)
  std::vector<double> glin[3];  // gamma_lin_u, _v, _eta
  std::vector<double> gsq[2];   // gamma_sq_u, _v
  std::vector<double> impl[3];
  std::vector<double> ubs, vbs, zbs;
};

struct Stream {
  int type, comp, is_const;
  double omega;
  double *d1 = nullptr, *d2 = nullptr;      // the record in use (device)
  double *rec[2] = {nullptr, nullptr};      // all records of parts 1 and 2 (device, optional)
  int nrec[2] = {0, 0};
};

struct DiagAcc {  // one time-averaging buffer (diagTask)
  double *buf = nullptr;
  double count = 0.;
};

struct Tracer {
  double kappa_h;
  double *CH[2] = {nullptr, nullptr};   // TRC_N0, TRC_N0p1 (rotated)
  double *G[3] = {nullptr, nullptr, nullptr};
  double *C = nullptr, *C0 = nullptr, *gamma = nullptr, *impl = nullptr;
  double *uhc = nullptr, *vhc = nullptr, *diff = nullptr;
  int n0 = 0, g0 = 0;
};

// Plain-old-data view of the device state handed to kernels by value.
struct Dev {
  int nx, ny, mode, qbf, barotropic, lateral_mixing, itt_is_zero;
  double dt, G, A, dLambda, dTheta, minD, tau_scale, RHO0, lbc;
  // the plain path's divisions by fixed divisors (divide.cuh); pdiv 0: the
  // division operator everywhere
  int pdiv;
  double r_dLambda, r_dTheta, AdT, r_AdT;  // 1/dLambda, 1/dTheta, A dTheta, 1/(A dTheta)
  const double *prow;                      // PROW_N per row (plain.cu)
  const double *rimpl[3];                  // 1 / impl_u, _v, _eta
  const int8_t *ocean[4];
  const double *cosl[4], *tanl[4], *f[4];
  double *Hg[4];  // H, H_u, H_v, H_eta on the device (H/H_u/H_v overwritten at itt=0 in linear modes)
  // state, N0 and N0p1
  double *u0, *v0, *eta0, *u1, *v1, *eta1;
  // increments: slot 1 (oldest) .. slot 3 (newest)
  double *Gu[3], *Gv[3], *Ge[3];
  double *D, *Dh, *Du, *Dv;
  double *edens, *pot, *zeta, *mu, *mv;
  double *pll, *plt, *lmu, *lmv;
  double *impl_u, *impl_v, *impl_e, *gsq_u, *gsq_v;
  double *Fx, *Fy, *Fe, *Fxc, *Fyc, *Fec;
  double *ubs, *vbs, *zbs;
};

}  // namespace swm

struct FusedState;
struct SorState;
struct IntegralScratch;
struct Trc32State;

struct swm_gpu_ctx {
  swm_gpu_config cfg;
  int device = -1;  // the CUDA device the context was created on
  int nx = 0, ny = 0;
  size_t n = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  swm::HostGrid hg;
  int stage = 0;  // 1 domain, 2 timestep_init, 3 damping, 4 forcing, 5 ic
  // device buffers
  int8_t *d_ocean[4] = {};
  double *d_cos[4] = {}, *d_tan[4] = {}, *d_f[4] = {}, *d_lat[4] = {};
  double *d_H[4] = {};
  double *u[2] = {}, *v[2] = {}, *eta[2] = {};
  int n0 = 0;  // index of the N0 time level
  double *Gu[3] = {}, *Gv[3] = {}, *Ge[3] = {};
  int g0 = 0;  // ring offset: increment slot k (1..3) lives in buffer (g0 + k - 1) % 3
  double *Dbuf[4] = {};  // own D arrays (FULLY_NONLINEAR)
  double *edens = nullptr, *pot = nullptr, *zeta = nullptr, *mu = nullptr, *mv = nullptr;
  double *pll = nullptr, *plt = nullptr, *lmu = nullptr, *lmv = nullptr;
  double *bh[4] = {};    // biharmonic scratch (first-pass pll, plt, lu, lv)
  double *ones = nullptr;
  // lateral-mixing coefficients of the plain path per row and mask case
  // (plain.cu k_latmix_tab_*): for up to two values of Ah, and the uv table
  double *latp[2] = {}, latp_ah[2] = {0., 0.}, *latuv = nullptr;
  // the plain path's fixed divisors and their reciprocals (plain_prepare):
  // per row A cos_eta, A cos_u dLambda, cos_H and the vorticity factors;
  // per point 1 / impl_u, _v, _eta; prow_ok: every divisor in div_fast's range
  double *prow = nullptr, *rimpl[3] = {};
  int *pdiv_bad = nullptr;
  bool pdiv = false, pdiv_ready = false;
  double *impl[3] = {}, *gsq[2] = {}, *glin[3] = {};
  double *F[3] = {}, *Fc[3] = {};
  double *ubs = nullptr, *vbs = nullptr, *zbs = nullptr;
  std::vector<swm::Stream> streams;
  std::vector<swm::Tracer> tracers;
  double *trc_coeff = nullptr;
  FusedState *fused = nullptr;
  SorState *sor = nullptr;
  IntegralScratch *integrals = nullptr;
  int integrals_shape[3] = {-1, 0, 0};  // k_integrals (FP64 state): tuned (0) or not (-1), threads, blocks
  Trc32State *trc32 = nullptr;      // tracers of the FP32 compensated path
  std::vector<swm::DiagAcc> diag;   // averaging buffers by slot
  std::vector<cudaEvent_t> async_ev;  // ring of events for swm_gpu_get_field_async
  std::atomic<int64_t> async_next{0};  // next ticket (read by a writer thread's waits)
  double *psi = nullptr, *psi_tmp = nullptr;  // streamfunction and its zonal sums
  double *rows_buf = nullptr;       // 2 x Ny staging rows of swm_gpu_set_stream_rows
  const swm::MonitorStep *mon = nullptr;  // the next FP32 pair step is a monitored step
  int64_t advances = 0;             // swm_gpu_advance calls (the rotation phase is advances mod 6)
  int march_rows = 0;                // rows per warp strip of the FP32 step kernel (0: not tuned yet)
  double march_S = 0.;               // rows per warp its tiles were cut for (cost target)
  double march_slow = 1.;            // masked-row cost its tiles were cut with
  int2 *march_tiles = nullptr;       // its tiles, one per warp (device)
  int march_blocks = 0;              // its blocks (tiles / 4)
  cudaGraphExec_t graph = nullptr;  // GRAPH_STEPS captured steps (swm_gpu_run)
  int64_t graph_launches = 0;       // kernels in one replay
  int graph_phase = -1;             // rotation phase (advances mod 6) the replay starts from
  swm::Dev dev() const;
};

namespace swm {
// setup.cu
int host_domain(swm_gpu_ctx *c, const double *H, const int8_t *H_missing);
void host_basic_state(swm_gpu_ctx *c, const double *psi);
void host_damping_add(swm_gpu_ctx *c, int term, int type, double value, double sl_length,
                      double sl_cutoff, int loc, const double *file_data);
void host_damping_finish(swm_gpu_ctx *c);

// plain.cu
int plain_diagnostics(swm_gpu_ctx *c, int64_t itt);
int plain_step(swm_gpu_ctx *c, int64_t itt);
int plain_prepare(swm_gpu_ctx *c);                // tables the plain step reads (before a capture)
int plain_forcing_update(swm_gpu_ctx *c, int64_t itt, int constant_part);
int plain_fill(swm_gpu_ctx *c, double *p, double value);
// tracer.cu
int tracer_init_coeffs(swm_gpu_ctx *c);
int tracer_step(swm_gpu_ctx *c, int64_t itt);
int tracer_advance(swm_gpu_ctx *c);
// fused.cu
int fused_prepare(swm_gpu_ctx *c);
int fused_step(swm_gpu_ctx *c, int64_t itt);
int fused_sync_state(swm_gpu_ctx *c);    // FP32 pair state -> FP64 buffers
int fused_load_state(swm_gpu_ctx *c);    // FP64 buffers -> FP32 pair state
int fused_refresh_wind(swm_gpu_ctx *c, int id);  // stream id's record changed
int stream_rows(swm_gpu_ctx *c, int id, const double *r1, const double *r2, const double *d1);
int integrals_to(swm_gpu_ctx *c, double *dst, double **where);  // dst: device or host-mapped
// swm_gpu_run_monitor on the FP32 pair path (one step kernel per step)
struct MonitorBufs {
  float *w[2];         // wind rows: the fused state's own, and the alternate
  int w_merid;         // the rows are the meridional ones
  double *partial[2];  // per-block sums of even and odd steps
  int nb;              // strip blocks of one step
  double *res;         // 3 x nsteps results when the caller's array is not mapped
};
bool monitor_fast(const swm_gpu_ctx *c);                 // the pair path is ready for it
bool monitor_rows_fast(const swm_gpu_ctx *c, int sid);   // stream sid's rows are converted in the step kernel
int monitor_buffers(swm_gpu_ctx *c, int64_t nsteps, int sid, bool rows, bool res, MonitorBufs *b);
int monitor_rows_first(swm_gpu_ctx *c, const double *rows_dev, float *w);
int monitor_finish(swm_gpu_ctx *c, const MonitorBufs &b, const double *partial, double *out);
int monitor_keep_rows(swm_gpu_ctx *c, const MonitorBufs &b, int last);
void fused_free(swm_gpu_ctx *c);
void integrals_free(swm_gpu_ctx *c);
// sor.cu
void sor_free(swm_gpu_ctx *c);
// api.cu
int async_record(swm_gpu_ctx *c, int64_t *ticket);  // ticket for the work queued so far
// diag.cu
int device_streamfunction(swm_gpu_ctx *c);
int diag_accumulate(swm_gpu_ctx *c, int slot, const double *f, int square, double w);
int diag_mean(swm_gpu_ctx *c, int slot, double *dev_out, double *count);
void diag_free(swm_gpu_ctx *c);
int stream_interp(swm_gpu_ctx *c, const double *rec, double *dst, int r0, int r1, double t, double t0, double t1);
// trc32.cu
bool trc32_active(const swm_gpu_ctx *c);
int trc32_add(swm_gpu_ctx *c, const std::vector<double> &CH, const std::vector<double> &C0,
              const std::vector<double> &gamma, const std::vector<double> &impl, double kappa);
int trc32_init(swm_gpu_ctx *c);
int trc32_step(swm_gpu_ctx *c, int64_t itt);
void trc32_advance(swm_gpu_ctx *c);
int trc32_export(swm_gpu_ctx *c, int t, int conc, double *dst);
void trc32_free(swm_gpu_ctx *c);
}  // namespace swm

#define SWM_LAUNCH_COUNT(c) ((c)->launches++)
