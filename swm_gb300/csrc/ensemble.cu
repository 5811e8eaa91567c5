// ensemble.cu -- an ensemble of basins of uneven sizes stepped together.
//
// Extension: the reference runs one basin per process.  Each member is an
// ordinary context on the FP32 compensated path, set up through the usual
// entry points; the ensemble gathers their kernel parameter blocks into a
// device table and cuts every member into warp tiles (strip of columns x
// group of rows).  One persistent launch per step drains a device queue of
// all members' tiles (k_march_ens), so small and large basins share the GPU
// without one launch per member.  The members' time levels and increment
// slots rotate in step, so the table holds one parameter block per member
// for each of the six phases of that rotation, and blocks of six steps replay
// one captured CUDA graph.  Per-member volume and energy sums are taken in
// FP64.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include "ctx.h"
#include "fused32.h"

using swm::P32;

namespace swm {

constexpr int ENS_PHASES = 6;  // lcm of the 2 levels and 3 increment slots
// tile candidates: rows per warp x masked-row cost
constexpr int ENS_TUNE_ROWS[] = {16, 24, 32, 48};
constexpr double ENS_TUNE_SLOW[] = {1.0, 1.7};

struct EnsInt {
  const float *uh, *ul, *vh, *vl, *eh, *el;
  const int8_t *oU, *oV, *oE;
  const double *cU, *cV, *cE;
  int nx, ny;
  double A2dLdT, G;
};

// one block per member: sums in FP64 of eta*area, 0.5*G*eta^2*area and the
// kinetic energy over the member's ocean points, as swm_gpu_integrals
__global__ void k_ens_integrals(const EnsInt *__restrict__ d, double *__restrict__ out) {
  __shared__ double red[3][256];
  const EnsInt q = d[blockIdx.x];
  double s0 = 0., s1 = 0., s2 = 0.;
  const int n = q.nx * q.ny;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int j = k / q.nx;
    const double ae = q.A2dLdT * q.cE[j], au = q.A2dLdT * q.cU[j], av = q.A2dLdT * q.cV[j];
    const double ee = (double)q.eh[k] + (double)q.el[k];
    const double uu = (double)q.uh[k] + (double)q.ul[k];
    const double vv = (double)q.vh[k] + (double)q.vl[k];
    if (q.oE[k]) {
      s0 += ee * ae;
      s1 += 0.5 * q.G * ee * ee * ae;
    }
    if (q.oU[k]) s2 += 0.5 * uu * uu * au;
    if (q.oV[k]) s2 += 0.5 * vv * vv * av;
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  red[2][threadIdx.x] = s2;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int r = 0; r < 3; r++) red[r][threadIdx.x] += red[r][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) out[3 * (size_t)blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

// monitored steps: one step's wind rows of every member (FP64: a staged copy,
// or the caller's pinned host array read in place) into each member's FP32
// row profile; the first thread also resets the step's queue head
__global__ void k_ens_rows(const double *__restrict__ rows, const int *__restrict__ row_member,
                           const int *__restrict__ row_off, float *const *__restrict__ w, int nrows,
                           int *__restrict__ queue_head) {
  grid_dep_wait();  // the previous step has finished reading the rows
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r == 0) *queue_head = 0;
  if (r >= nrows || !rows) return;
  const int i = row_member[r];
  w[i][r - row_off[i]] = (float)rows[r];
}

// monitored steps: the integrals of every member from its tiles' sums, one
// warp per member: lane l adds the member's tiles l, l + 32, ... (in queue
// order), then a shuffle tree in fixed order; out may be pinned host memory
__global__ void k_ens_tile_sums(const double *__restrict__ partial, const int *__restrict__ tile_off,
                                const int *__restrict__ tiles_of, const double *__restrict__ G, int n,
                                double *__restrict__ out) {
  grid_dep_wait();  // the step's tile sums are written
  const int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (i >= n) return;  // whole warps leave together
  double s[4] = {0., 0., 0., 0.};
  for (int k = tile_off[i] + lane; k < tile_off[i + 1]; k += 32) {
    const double *q = partial + 4 * (size_t)tiles_of[k];
    s[0] += q[0];
    s[1] += q[1];
    s[2] += q[2];
    s[3] += q[3];
  }
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 4; c++) s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
  if (lane == 0) {
    out[3 * (size_t)i] = s[0];
    out[3 * (size_t)i + 1] = 0.5 * G[i] * s[1];
    out[3 * (size_t)i + 2] = 0.5 * (s[2] + s[3]);
  }
}

// device tables of the monitored steps, built on their first use
struct EnsMonitor {
  int nrows = 0;                 // rows of all members: the doubles of one step's wind rows
  std::vector<int> row_off;      // first row of each member in a step's rows
  std::vector<int> wind_sid;     // each member's row-profile wind stream
  double *rows[2] = {nullptr, nullptr};  // one step's rows, alternating
  int *row_member = nullptr, *d_row_off = nullptr;
  float **w = nullptr;           // each member's FP32 wind rows
  const float2 **areas = nullptr;
  double *partial = nullptr;     // 4 per tile
  int *tile_off = nullptr, *tiles_of = nullptr;
  double *G = nullptr;
  double *res = nullptr;         // 3 per member
  bool has_rows = false;         // every member has a row-profile zonal wind stream
};

}  // namespace swm

struct swm_gpu_ensemble {
  std::vector<swm_gpu_ctx *> m;
  int device = -1;  // the members' device
  int mix = 0, rows = 16, phase = 0, graph_phase = -1;
  double slow = 1.;  // masked-row cost the tiles were cut with
  bool std_cfg = false;  // all members in the step kernel's common configuration
  int pf = 1;            // the step kernel's prefetch level for the members' state
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<cudaEvent_t> ev;
  P32 *tab = nullptr;  // [ENS_PHASES][n]
  int4 *tiles = nullptr;  // {member, strip, first row, rows}, costliest first
  int ntiles = 0;
  int *next = nullptr;  // queue heads, one per phase
  cudaGraphExec_t graph = nullptr;
  int64_t launches = 0, graph_launches = 0;
  swm::EnsInt *d_int = nullptr;
  double *d_out = nullptr;
  std::vector<int4> htiles;  // host copy of the tiles in queue order
  swm::EnsMonitor *mon = nullptr;
};

namespace {

using namespace swm;

int join_members(swm_gpu_ensemble *e) {  // ensemble stream waits for every member stream
  for (size_t i = 0; i < e->m.size(); i++) {
    SWM_CK(cudaEventRecord(e->ev[i], e->m[i]->stream));
    SWM_CK(cudaStreamWaitEvent(e->stream, e->ev[i], 0));
  }
  return SWM_GPU_OK;
}

int release_members(swm_gpu_ensemble *e) {  // member streams wait for the ensemble stream
  SWM_CK(cudaEventRecord(e->done, e->stream));
  for (auto *c : e->m) SWM_CK(cudaStreamWaitEvent(c->stream, e->done, 0));
  return SWM_GPU_OK;
}

// host side of one ensemble step: every member's level and slot offsets
// advance as swm_gpu_step + swm_gpu_advance would advance them
int rotate_members(swm_gpu_ensemble *e, int64_t itt) {
  for (auto *c : e->m) {
    int n0, g0;
    fused_indices(c, &n0, &g0);
    fused_set_indices(c, 1 - n0, (g0 + 1) % 3);
    int rc = swm_gpu_advance(c, itt);
    if (rc != SWM_GPU_OK) return rc;
  }
  e->phase = (e->phase + 1) % ENS_PHASES;
  return SWM_GPU_OK;
}

// the device address of host memory the GPU can read in place (pinned and
// mapped), or null
const void *mapped_device_pointer(const void *host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();  // clear the error of an unregistered pointer
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int ens_step(swm_gpu_ensemble *e, int64_t itt, const EnsInteg *mi = nullptr, bool reset_head = true) {
  const size_t n = e->m.size();
  if (reset_head) SWM_CK(cudaMemsetAsync(e->next + e->phase, 0, sizeof(int), e->stream));
  int rc = march_ens_launch(e->mix, e->std_cfg, e->pf, e->tab + (size_t)e->phase * n, e->tiles, e->ntiles,
                            e->next + e->phase, e->stream, mi);
  if (rc != SWM_GPU_OK) return rc;
  e->launches++;
  return rotate_members(e, itt);
}

int ens_capture(swm_gpu_ensemble *e, int64_t itt0) {
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  const int phase0 = e->phase;
  const int64_t l0 = e->launches;
  SWM_CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  // each phase has its own queue head: one reset of all of them serves the
  // graph's six steps
  cudaError_t me = cudaMemsetAsync(e->next, 0, ENS_PHASES * sizeof(int), e->stream);
  int rc = SWM_GPU_OK;
  if (me != cudaSuccess) {
    set_error(std::string("swm_gpu_ensemble_run: cudaMemsetAsync: ") + cudaGetErrorString(me));
    rc = SWM_GPU_ECUDA;
  }
  for (int s = 1; s <= ENS_PHASES && rc == SWM_GPU_OK; s++) rc = ens_step(e, itt0 + s, nullptr, false);
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
  e->graph_launches = e->launches - l0;
  e->launches = l0;
  if (rc != SWM_GPU_OK || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc != SWM_GPU_OK) return rc;
    set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    return SWM_GPU_ECUDA;
  }
  SWM_REQUIRE(e->phase == phase0, "swm_gpu_ensemble_run: phase cycle mismatch");
  ce = cudaGraphInstantiate(&e->graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) {
    e->graph = nullptr;
    set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
    return SWM_GPU_ECUDA;
  }
  e->graph_phase = phase0;
  return SWM_GPU_OK;
}

// the monitored steps' device tables (first use)
int ens_monitor_setup(swm_gpu_ensemble *e) {
  if (e->mon) return SWM_GPU_OK;
  const int n = (int)e->m.size();
  EnsMonitor *M = new EnsMonitor();
  e->mon = M;
  std::vector<float *> w(n);
  std::vector<const float2 *> areas(n);
  std::vector<double> G(n);
  std::vector<int> row_member;
  M->has_rows = true;
  M->row_off.resize(n);
  M->wind_sid.assign(n, -1);
  for (int i = 0; i < n; i++) {
    swm_gpu_ctx *c = e->m[i];
    int rc = fused_monitor_inputs(c, SWM_CMP_ZONAL, &w[i], &areas[i]);
    if (rc != SWM_GPU_OK) return rc;
    for (size_t k = 0; k < c->streams.size(); k++) {
      const Stream &st = c->streams[k];
      if (st.type == SWM_FRC_WIND && st.comp == SWM_CMP_ZONAL && !st.is_const) {
        M->wind_sid[i] = (int)k;
        break;
      }
    }
    M->has_rows = M->has_rows && w[i] && M->wind_sid[i] >= 0;
    G[i] = c->cfg.G;
    M->row_off[i] = M->nrows;
    row_member.insert(row_member.end(), c->ny, i);
    M->nrows += c->ny;
  }
  // each member's tiles in queue order (the order its sums are added in)
  std::vector<int> tile_off(n + 1, 0), tiles_of(e->ntiles);
  for (const int4 &t : e->htiles) tile_off[t.x + 1]++;
  for (int i = 0; i < n; i++) tile_off[i + 1] += tile_off[i];
  std::vector<int> fill(tile_off.begin(), tile_off.end() - 1);
  for (int t = 0; t < e->ntiles; t++) tiles_of[fill[e->htiles[t].x]++] = t;
  auto up = [&](void **dst, const void *src, size_t bytes) {
    if (cudaMalloc(dst, bytes) != cudaSuccess) return SWM_GPU_ENOMEM;
    if (src && cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return SWM_GPU_ECUDA;
    return SWM_GPU_OK;
  };
  int rc = SWM_GPU_OK;
  for (int b = 0; b < 2 && rc == SWM_GPU_OK; b++) rc = up((void **)&M->rows[b], nullptr, M->nrows * sizeof(double));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->row_member, row_member.data(), M->nrows * sizeof(int));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->d_row_off, M->row_off.data(), n * sizeof(int));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->w, w.data(), n * sizeof(float *));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->areas, areas.data(), n * sizeof(float2 *));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->partial, nullptr, 4 * (size_t)e->ntiles * sizeof(double));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->tile_off, tile_off.data(), (n + 1) * sizeof(int));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->tiles_of, tiles_of.data(), e->ntiles * sizeof(int));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->G, G.data(), n * sizeof(double));
  if (rc == SWM_GPU_OK) rc = up((void **)&M->res, nullptr, 3 * (size_t)n * sizeof(double));
  if (rc != SWM_GPU_OK) set_error("swm_gpu_ensemble_run_monitor: device tables could not be set up");
  return rc;
}

void ens_free(swm_gpu_ensemble *e) {
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  cudaFree(e->tab);
  cudaFree(e->tiles);
  cudaFree(e->next);
  cudaFree(e->d_int);
  cudaFree(e->d_out);
  if (EnsMonitor *m = e->mon) {
    cudaFree(m->rows[0]);
    cudaFree(m->rows[1]);
    cudaFree(m->row_member);
    cudaFree(m->d_row_off);
    cudaFree(m->w);
    cudaFree(m->areas);
    cudaFree(m->partial);
    cudaFree(m->tile_off);
    cudaFree(m->tiles_of);
    cudaFree(m->G);
    cudaFree(m->res);
    delete m;
  }
  for (auto ev : e->ev) cudaEventDestroy(ev);
  if (e->done) cudaEventDestroy(e->done);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

}  // namespace

extern "C" {

int swm_gpu_ensemble_create(swm_gpu_ctx *const *members, int n, swm_gpu_ensemble **out) {
  SWM_REQUIRE(members && n > 0 && out, "swm_gpu_ensemble_create: bad arguments");
  *out = nullptr;
  SWM_REQUIRE(members[0], "swm_gpu_ensemble_create: members must be initialised");
  for (int i = 1; i < n; i++)
    SWM_REQUIRE(members[i] && members[i]->device == members[0]->device,
                "swm_gpu_ensemble_create: members must live on one device");
  SWM_ON_DEVICE(members[0]->device);
  int n0 = -1, g0 = -1, mix = -1;
  for (int i = 0; i < n; i++) {
    swm_gpu_ctx *c = members[i];
    SWM_REQUIRE(c && c->stage >= 5, "swm_gpu_ensemble_create: members must be initialised");
    SWM_REQUIRE(c->cfg.path == SWM_PATH_FUSED_FP32C, "swm_gpu_ensemble_create: members must use SWM_PATH_FUSED_FP32C");
    SWM_REQUIRE(c->tracers.empty(), "swm_gpu_ensemble_create: members with tracers are not batched");
    SWM_REQUIRE(c->cfg.mode != SWM_MODE_LIN_MEAN,
                "swm_gpu_ensemble_create: LINEARISED_MEAN_STATE members are stepped on their own");
    for (const Stream &st : c->streams)
      SWM_REQUIRE(st.type != SWM_FRC_OSC, "swm_gpu_ensemble_create: members with oscillating forcing are stepped "
                                          "on their own");
    SWM_REQUIRE(c->ny < (1 << 23), "swm_gpu_ensemble_create: member too large for a tile index");
    if (!c->march_rows) c->march_rows = 16;  // the ensemble tunes its own strip rows
    int rc = fused_prepare(c);
    if (rc != SWM_GPU_OK) return rc;
    // the batched step reads each member's forcing fields as they are; a
    // member whose forcing fields change every step is stepped on its own
    SWM_REQUIRE(!fused_dynamic_forcing(c), "swm_gpu_ensemble_create: members with time-dependent forcing other "
                                           "than the nonlinear wind stress are stepped on their own");
    int a, b;
    fused_indices(c, &a, &b);
    int mx = c->cfg.lateral_mixing ? (c->cfg.mixing_kind == SWM_MIX_BIHARMONIC ? 2 : 1) : 0;
    if (i == 0) { n0 = a; g0 = b; mix = mx; }
    SWM_REQUIRE(a == n0 && b == g0, "swm_gpu_ensemble_create: members must be at the same step");
    SWM_REQUIRE(mx == mix, "swm_gpu_ensemble_create: members must share the lateral-mixing kind");
  }
  swm_gpu_ensemble *e = new swm_gpu_ensemble();
  e->m.assign(members, members + n);
  e->device = members[0]->device;
  e->mix = mix;
  auto fail = [&](int rc) { ens_free(e); return rc; };
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming) != cudaSuccess) {
    set_error("swm_gpu_ensemble_create: stream or event creation failed");
    return fail(SWM_GPU_ECUDA);
  }
  e->ev.resize(n);
  for (int i = 0; i < n; i++)
    if (cudaEventCreateWithFlags(&e->ev[i], cudaEventDisableTiming) != cudaSuccess) {
      set_error("swm_gpu_ensemble_create: event creation failed");
      return fail(SWM_GPU_ECUDA);
    }
  // parameter blocks for the six phases (AB3 weights: the table serves itt >= 3)
  std::vector<P32> tab((size_t)ENS_PHASES * n);
  for (int k = 0; k < ENS_PHASES; k++)
    for (int i = 0; i < n; i++) {
      fused_set_indices(members[i], (n0 + k) % 2, (g0 + k) % 3);
      make_p32(members[i], 3, tab[(size_t)k * n + i]);
    }
  for (int i = 0; i < n; i++) fused_set_indices(members[i], n0, g0);
  e->std_cfg = true;
  for (const P32 &q : tab) e->std_cfg = e->std_cfg && march_std_params(q);
  size_t points = 0;
  for (int i = 0; i < n; i++) points += (size_t)members[i]->nx * members[i]->ny;
  e->pf = march_prefetch_level(points, false);
  for (int i = 0; i < n && e->pf == 3; i++)
    if (members[i]->nx < RING_MIN_NX) e->pf = 2;  // the row ring wants basins RING_MIN_NX wide
  for (P32 &q : tab) q.pf = e->pf;
  // Tiles: every member's strips cut into row groups of equal estimated
  // cost (as the single-basin step kernel's tiles), all members' tiles in
  // one queue with the short remainder groups last, so the queue ends on
  // small tiles and the warps finish close together.  Candidates: rows per
  // warp x masked-row cost, timed below.
  std::vector<std::vector<uint8_t>> fast(n);
  for (int i = 0; i < n; i++) {
    const uint16_t *m16 = fused_mask_words(members[i]);
    SWM_REQUIRE(m16, "swm_gpu_ensemble_create: member has no FP32 pair state");
    fast[i] = march_fast_rows(mix, members[i]->nx, members[i]->ny, m16);
  }
  std::vector<std::pair<double, double>> cand;
  const double s_env = march_rows_override_f(), w_env = march_slow_override();
  for (int S : ENS_TUNE_ROWS)
    for (double w : ENS_TUNE_SLOW) {
      const std::pair<double, double> q(s_env > 0. ? s_env : S, w_env > 0. ? w_env : w);
      if (std::find(cand.begin(), cand.end(), q) == cand.end()) cand.push_back(q);
    }
  std::vector<std::vector<int4>> lists(cand.size());
  size_t maxn = 0;
  for (size_t r = 0; r < cand.size(); r++) {
    std::vector<std::pair<double, int4>> t;
    for (int i = 0; i < n; i++) {
      const int ny = members[i]->ny;
      for (const int2 g : march_tiles_cut(fast[i], ny, cand[r].first, cand[r].second))
        if (g.y & 255)
          t.push_back({march_tile_cost(fast[i], ny, g, cand[r].second), make_int4(i, g.x, g.y >> 8, g.y & 255)});
    }
    // full groups (cost within 3/4 of the target) first, in their natural
    // order: vertically adjacent groups of a strip go to warps at about the
    // same time and share their look-ahead rows in L2; the short remainders
    // after them, costliest first
    const double full = 0.75 * (cand[r].first + 3.0);
    std::stable_sort(t.begin(), t.end(), [full](const std::pair<double, int4> &a, const std::pair<double, int4> &b) {
      const bool fa = a.first >= full, fb = b.first >= full;
      if (fa != fb) return fa;
      return !fa && a.first > b.first;
    });
    for (auto &q : t) lists[r].push_back(q.second);
    maxn = std::max(maxn, lists[r].size());
  }
  if (cudaMalloc((void **)&e->tab, tab.size() * sizeof(P32)) != cudaSuccess ||
      cudaMemcpy(e->tab, tab.data(), tab.size() * sizeof(P32), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMalloc((void **)&e->next, ENS_PHASES * sizeof(int)) != cudaSuccess ||
      cudaMalloc((void **)&e->d_int, n * sizeof(EnsInt)) != cudaSuccess ||
      cudaMalloc((void **)&e->d_out, 3 * (size_t)n * sizeof(double)) != cudaSuccess) {
    set_error("swm_gpu_ensemble_create: device allocation failed");
    return fail(SWM_GPU_ENOMEM);
  }
  // tiles by timing the ensemble step at the current phase (the step
  // rewrites level N0p1 and slot 3 only, which the first real step rewrites)
  if (cudaMalloc((void **)&e->tiles, maxn * sizeof(int4)) != cudaSuccess) {
    set_error("swm_gpu_ensemble_create: tile list allocation failed");
    return fail(SWM_GPU_ENOMEM);
  }
  if (join_members(e) != SWM_GPU_OK) return fail(SWM_GPU_ECUDA);
  int best = 0, uploaded = -1;
  std::vector<int> idx(cand.size());
  for (size_t r = 0; r < idx.size(); r++) idx[r] = (int)r;
  int rc = SWM_GPU_OK;
  if (cand.size() > 1)
    rc = march_pick_rows(e->stream, 3, idx, [&](int r) {
      if (uploaded != r) {
        cudaMemcpyAsync(e->tiles, lists[r].data(), lists[r].size() * sizeof(int4), cudaMemcpyHostToDevice,
                        e->stream);
        uploaded = r;
      }
      cudaMemsetAsync(e->next, 0, sizeof(int), e->stream);
      march_ens_launch(mix, e->std_cfg, e->pf, e->tab, e->tiles, (int)lists[r].size(), e->next, e->stream);
    }, &best);
  if (rc != SWM_GPU_OK) return fail(rc);
  if (cudaMemcpyAsync(e->tiles, lists[best].data(), lists[best].size() * sizeof(int4), cudaMemcpyHostToDevice,
                      e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess) {
    set_error("swm_gpu_ensemble_create: tile list upload failed");
    return fail(SWM_GPU_ECUDA);
  }
  e->ntiles = (int)lists[best].size();
  e->htiles = lists[best];
  e->rows = (int)cand[best].first;
  e->slow = cand[best].second;
  if (release_members(e) != SWM_GPU_OK) return fail(SWM_GPU_ECUDA);
  *out = e;
  return SWM_GPU_OK;
}

int swm_gpu_ensemble_destroy(swm_gpu_ensemble *e) {
  SWM_ON_DEVICE(e ? e->device : -1);
  if (e) ens_free(e);
  return SWM_GPU_OK;
}

int swm_gpu_ensemble_run(swm_gpu_ensemble *e, int64_t itt0, int64_t nsteps) {
  SWM_ON_DEVICE(e ? e->device : -1);
  SWM_REQUIRE(e && nsteps >= 0, "swm_gpu_ensemble_run: bad arguments");
  int64_t s = 1;
  // Adams-Bashforth start-up steps (itt 1, 2): each member on its own stream
  for (; s <= nsteps && itt0 + s < 3; s++) {
    for (auto *c : e->m) {
      int rc = swm_gpu_step(c, itt0 + s);
      if (rc == SWM_GPU_OK) rc = swm_gpu_advance(c, itt0 + s);
      if (rc != SWM_GPU_OK) return rc;
    }
    e->phase = (e->phase + 1) % ENS_PHASES;
  }
  if (s > nsteps) return SWM_GPU_OK;
  int rc = join_members(e);
  if (rc != SWM_GPU_OK) return rc;
  while (s <= nsteps) {
    const int64_t itt = itt0 + s;
    if (nsteps - s + 1 >= ENS_PHASES) {
      if (!e->graph) {
        rc = ens_capture(e, itt - 1);
        if (rc != SWM_GPU_OK) return rc;
      }
      if (e->phase == e->graph_phase) {
        SWM_CK(cudaGraphLaunch(e->graph, e->stream));
        e->launches += e->graph_launches;
        s += ENS_PHASES;
        continue;
      }
    }
    rc = ens_step(e, itt);
    if (rc != SWM_GPU_OK) return rc;
    s++;
  }
  rc = release_members(e);
  if (rc != SWM_GPU_OK) return rc;
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

int swm_gpu_ensemble_run_monitor(swm_gpu_ensemble *e, int64_t itt0, int64_t nsteps, const double *rows,
                                 double *out) {
  SWM_ON_DEVICE(e ? e->device : -1);
  SWM_REQUIRE(e && nsteps >= 0 && out, "swm_gpu_ensemble_run_monitor: bad arguments");
  int rc = ens_monitor_setup(e);
  if (rc != SWM_GPU_OK) return rc;
  EnsMonitor *M = e->mon;
  SWM_REQUIRE(!rows || M->has_rows,
              "swm_gpu_ensemble_run_monitor: rows need a time-dependent row-profile zonal wind stress in every member");
  const size_t n = e->m.size();
  // pinned (host-mapped) arrays are read and written in place by the kernels
  const double *rows_dev = rows ? static_cast<const double *>(mapped_device_pointer(rows)) : nullptr;
  double *out_dev = static_cast<double *>(const_cast<void *>(mapped_device_pointer(out)));
  bool joined = false;
  for (int64_t s = 0; s < nsteps; s++) {
    const int64_t itt = itt0 + s + 1;
    const double *rs = rows ? rows + (size_t)s * M->nrows : nullptr;
    double *os = out + 3 * n * (size_t)s;
    if (itt < 3) {
      // Adams-Bashforth start-up: each member on its own stream, as
      // swm_gpu_ensemble_run does, then swm_gpu_ensemble_integrals
      for (size_t i = 0; i < n; i++) {
        swm_gpu_ctx *c = e->m[i];
        if (rs) rc = swm_gpu_set_stream_rows(c, M->wind_sid[i], rs + M->row_off[i], nullptr);
        if (rc == SWM_GPU_OK) rc = swm_gpu_step(c, itt);
        if (rc == SWM_GPU_OK) rc = swm_gpu_advance(c, itt);
        if (rc != SWM_GPU_OK) return rc;
      }
      e->phase = (e->phase + 1) % ENS_PHASES;
      rc = swm_gpu_ensemble_integrals(e, os);
      if (rc != SWM_GPU_OK) return rc;
      continue;
    }
    if (!joined) {
      rc = join_members(e);
      if (rc != SWM_GPU_OK) return rc;
      joined = true;
    }
    const double *rd = nullptr;  // the rows as the device reads them
    if (rs) {
      if (rows_dev) {
        rd = rows_dev + (size_t)s * M->nrows;
      } else {
        double *d = M->rows[s & 1];
        SWM_CK(cudaMemcpyAsync(d, rs, M->nrows * sizeof(double), cudaMemcpyHostToDevice, e->stream));
        rd = d;
      }
    }
    // the three kernels of a monitored step are launched programmatically:
    // each may be launched while its predecessor finishes and waits for it
    // on the device (grid_dep_wait), so no launch latency separates them
    SWM_CK(launch_programmatic(k_ens_rows, dim3(rd ? (M->nrows + 255) / 256 : 1), dim3(256), e->stream, rd,
                               (const int *)M->row_member, (const int *)M->d_row_off, (float *const *)M->w,
                               M->nrows, e->next + e->phase));
    e->launches++;
    const EnsInteg mi{M->areas, M->partial};
    rc = ens_step(e, itt, &mi, false);
    if (rc != SWM_GPU_OK) return rc;
    double *od = out_dev ? out_dev + 3 * n * (size_t)s : M->res;
    SWM_CK(launch_programmatic(k_ens_tile_sums, dim3((unsigned)((32 * n + 127) / 128)), dim3(128), e->stream,
                               (const double *)M->partial, (const int *)M->tile_off, (const int *)M->tiles_of,
                               (const double *)M->G, (int)n, od));
    e->launches++;
    if (!out_dev) SWM_CK(cudaMemcpyAsync(os, M->res, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  }
  if (joined) {
    rc = release_members(e);
    if (rc != SWM_GPU_OK) return rc;
  }
  SWM_CK(cudaGetLastError());
  SWM_CK(cudaStreamSynchronize(e->stream));
  return SWM_GPU_OK;
}

int swm_gpu_ensemble_integrals(swm_gpu_ensemble *e, double *out) {
  SWM_ON_DEVICE(e ? e->device : -1);
  SWM_REQUIRE(e && out, "swm_gpu_ensemble_integrals: bad arguments");
  const size_t n = e->m.size();
  std::vector<EnsInt> d(n);
  for (size_t i = 0; i < n; i++) {
    swm_gpu_ctx *c = e->m[i];
    const float *lv[6];
    fused_pair_level(c, lv);
    EnsInt &q = d[i];
    q.uh = lv[0]; q.ul = lv[1]; q.vh = lv[2]; q.vl = lv[3]; q.eh = lv[4]; q.el = lv[5];
    q.oU = c->d_ocean[GU]; q.oV = c->d_ocean[GV]; q.oE = c->d_ocean[GE];
    q.cU = c->d_cos[GU]; q.cV = c->d_cos[GV]; q.cE = c->d_cos[GE];
    q.nx = c->nx; q.ny = c->ny;
    q.A2dLdT = c->cfg.A * c->cfg.A * c->hg.dLambda * c->hg.dTheta;
    q.G = c->cfg.G;
  }
  int rc = join_members(e);
  if (rc != SWM_GPU_OK) return rc;
  SWM_CK(cudaMemcpyAsync(e->d_int, d.data(), n * sizeof(EnsInt), cudaMemcpyHostToDevice, e->stream));
  k_ens_integrals<<<(unsigned)n, 256, 0, e->stream>>>(e->d_int, e->d_out);
  e->launches++;
  SWM_CK(cudaGetLastError());
  SWM_CK(cudaMemcpyAsync(out, e->d_out, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  SWM_CK(cudaStreamSynchronize(e->stream));
  return SWM_GPU_OK;
}

int swm_gpu_ensemble_synchronize(swm_gpu_ensemble *e) {
  SWM_ON_DEVICE(e ? e->device : -1);
  SWM_REQUIRE(e, "swm_gpu_ensemble_synchronize: null ensemble");
  SWM_CK(cudaStreamSynchronize(e->stream));
  return march_ring_check();
}

void *swm_gpu_ensemble_stream(swm_gpu_ensemble *e) { return e ? (void *)e->stream : nullptr; }

int64_t swm_gpu_ensemble_launch_count(swm_gpu_ensemble *e) { return e ? e->launches : -1; }

int swm_gpu_ensemble_rows(swm_gpu_ensemble *e) { return e ? e->rows : 0; }

}  // extern "C"
