// fused32.h -- parameter block of the FP32 compensated step kernel (march.cu).
#pragma once
#include <functional>
#include <vector>
#include "ctx.h"

namespace swm {

// per-row factors (computed in FP64 on the host, stored as binary32)
enum {
  Q_CV, Q_DCV, Q_CU, Q_DCU, Q_FH, Q_RE_DL, Q_RE_DT, Q_RU_DL, Q_RV_DL, Q_RH_DL, Q_INV_CH,
  Q_PC0, Q_HC0, Q_TE, Q_TH, Q_TU, Q_TV, Q_NR
};

// The step kernel reads the factors of rows J, J-1 and J-2 in the iteration
// that loads row J.  Record J holds exactly those, as float4 groups in the
// order of the code that uses them, so an iteration issues a few vector
// loads of one warp-uniform address instead of a load per factor:
//   A {RH_DL, CU, DCU, INV_CH} (J)          relative vorticity and PV
//   G {FH (J), 0, 0, 0}                     PV
//   B {TE, PC0 (J-1), TH, HC0 (J)}          first stress pass
//   C {TU, RU_DL, TV, RV_DL} (J-1)          lu1, lv1
//   D {TE, PC0 (J-2), TH, HC0 (J-1)}        second (or the only) stress pass
//   E {CV, DCV (J-1), RE_DL, RE_DT (J-2)}   eta tendency
//   F {RU_DL, TU, TV, RV_DL} (J-2)          u and v tendencies
enum { REC_A, REC_G, REC_B, REC_C, REC_D, REC_E, REC_F, REC_N };
std::vector<float> fp32c_records(const swm_gpu_ctx *c);  // REC_N * 4 floats per row

struct P32 {
  int nx, ny, nl, mix, qbf, barotropic, has_F, impl_uniform, gsq_uniform, wind_x, wind_y, wind_rows, has_mode;
  int pf;  // L2 prefetch level of the two-column step kernel (march_prefetch_level), set at launch
  float dt, G, minD, lbc, q1, ts_rho, Ah, bih;
  float ab0, ab1, ab2;
  float impl_s[3], dp_s[3], gsq_s[2];
  const uint16_t *mask16;
  const float *dp[3];
  const float *He, *Hu, *Hv;
  const float4 *rec;  // per-iteration factor records, REC_N per row
  const float *impl[3], *gsq[2];
  const float *Fx, *Fy, *Fe;
  const float *wx, *wy;
  const float *uh0, *ul0, *vh0, *vl0, *eh0, *el0;
  float *uh1, *ul1, *vh1, *vl1, *eh1, *el1;
  const float *Gu1, *Gu2, *Gv1, *Gv2, *Ge1, *Ge2;
  float *Gu3, *Gv3, *Ge3;
};

#ifdef __CUDACC__
// (hi, lo) binary32 accumulator: TwoSum keeps the rounding error of every
// addition, so a sum carries about 46 bits.  Used for domain sums of the
// pair state, where FP64 arithmetic per point would tie a kernel to the
// FP64 pipe.
struct F2 {
  float h = 0.f, l = 0.f;
  __device__ __forceinline__ void add(float a, float b) {  // += a + b, |b| << |a|
    const float s = h + a, bb = s - h;
    l += ((h - (s - bb)) + (a - bb)) + b;
    h = s;
  }
  // += (a.x + a.y) * (r.h + r.l): TwoProd of the high parts plus the cross
  // terms (the low-low product is below the pair's precision)
  __device__ __forceinline__ void add_prod(float2 a, const F2 &r) {
    const float p = a.x * r.h;
    add(p, fmaf(a.x, r.h, -p) + fmaf(a.x, r.l, a.y * r.h));
  }
  __device__ __forceinline__ double value() const { return (double)h + (double)l; }
};

// Programmatic dependent launch: a kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may start before its
// predecessor on the stream has finished; grid_dep_wait() returns once the
// predecessor has completed and its writes are visible (at once for a kernel
// launched the ordinary way).  grid_dep_trigger() lets the successor launch.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ask L2 for the line holding a (no register is written, nothing waits)
__device__ __forceinline__ void prefetch_l2(const void *a) { asm volatile("prefetch.global.L2 [%0];" ::"l"(a)); }

// the square of the pair (x, xl) as a pair: TwoProd of the high parts plus
// the cross term (xl^2 is below the pair's precision)
__device__ __forceinline__ void sq_pair(float x, float xl, float &p, float &e) {
  p = x * x;
  e = fmaf(x, x, -p) + 2.f * x * xl;
}
#endif

// Monitored steps of the pair state (k_march<MIX, true>).  The strip blocks
// (blockIdx.x >= 1) also sum the new state of their ocean points times the
// cell areas: per block eta*area, eta^2*area, u^2*area_u, v^2*area_v into
// partial[q * nb + b] (nb strip blocks).  Block 0 does the step's side jobs
// while they run: it converts the next step's wind rows (host-mapped FP64)
// into next_w, and it finishes the previous step's sums (prev_partial) into
// prev_out[3] = {sum eta*area, 0.5 G sum eta^2*area, 0.5 (sum u^2*area_u +
// sum v^2*area_v)}, in the order k_march_integrals_final uses.  prev_out may
// be host-mapped memory.
struct MarchInteg {
  const float2 *area;  // (hi, lo) cell areas of the u, v, eta rows, 3 x ny
  double *partial;
  const double *prev_partial;  // null: nothing to finish
  double *prev_out;
  const double *next_rows;  // null: no rows to convert
  float *next_w;
  double G;
  int ny;
  int programmatic;  // launch as a programmatic dependent of the stream's previous kernel
};

// one monitored step as swm_gpu_run_monitor sets it up for the step kernel
struct MonitorStep {
  float *w_now;   // wind rows the step reads (null: the fused state's own)
  int w_merid;    // w_now replaces the meridional rows (else the zonal)
  double *partial;
  const double *prev_partial;
  double *prev_out;
  const double *next_rows;
  float *next_w;
};

// the integrals of one monitored step from its per-block sums (nb strip
// blocks) into out[3]
void march_integrals_final(const double *partial, int nb, double G, double *out, cudaStream_t st);

// cudaLaunchKernelEx with programmatic stream serialisation (see grid_dep_wait)
template <typename... KArgs, typename... Args>
cudaError_t launch_programmatic(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
// the step kernel's tiles (device) and blocks
struct MarchGrid {
  const int2 *tiles;
  int blocks;
};
std::vector<int2> march_tiles(int mix, int nx, int ny, const uint16_t *m16, double S, double slow);
std::vector<uint8_t> march_fast_rows(int mix, int nx, int ny, const uint16_t *m16);
std::vector<int2> march_tiles_cut(const std::vector<uint8_t> &fast, int ny, double S, double slow);
double march_tile_cost(const std::vector<uint8_t> &fast, int ny, int2 t, double slow);
const uint16_t *fused_mask_words(const swm_gpu_ctx *c);  // host copy, FP32 pair path
int march_default_tiles(swm_gpu_ctx *c, const P32 &p, const uint16_t *m16, int S);

// candidate rows per warp strip of the step kernel
constexpr int MARCH_NROWS = 4;
constexpr int MARCH_ROWS[MARCH_NROWS] = {8, 16, 24, 32};

std::vector<double> fp32c_rows(const swm_gpu_ctx *c);
void make_p32(const swm_gpu_ctx *c, int64_t itt, P32 &p);
void march_launch(swm_gpu_ctx *c, const P32 &p, const MarchGrid &g, const MarchInteg *mi = nullptr);
int march_tile_cols(int mix);          // columns a warp strip updates
int march_rows_override();             // SWM_GB300_MARCH_S, 0 when unset
double march_rows_override_f();        // the same, quarters allowed
double march_slow_override();         // SWM_GB300_MARCH_SLOW, 0 when unset
int march_pick_rows(cudaStream_t st, int reps, const std::vector<int> &cands, const std::function<void(int)> &launch,
                    int *best);
int march_autotune(swm_gpu_ctx *c, const P32 &p, const uint16_t *m16);
void fused_indices(const swm_gpu_ctx *c, int *n0, int *g0);
void fused_set_indices(swm_gpu_ctx *c, int n0, int g0);
void fused_pair_level(const swm_gpu_ctx *c, const float *out[6]);
void fused_static(const swm_gpu_ctx *c, const float **He, const uint16_t **mask16, const float **Fe);
// one launch of the ensemble step: tiles {member, strip, first row, rows}
// std_cfg: every member's parameter block is of the common configuration
// (march_std_params), so the kernel's specialised instance serves them
// pf: the step kernel's prefetch level (march_prefetch_level)
// mi: a monitored step (the sums of k_march_ens's INTEG instance), or null
struct EnsInteg {
  const float2 *const *areas;  // per member: (hi, lo) cell areas of the u, v, eta rows, 3 x ny
  double *partial;             // 4 sums per tile
};
int march_ens_launch(int mix, bool std_cfg, int pf, const P32 *tab, const int4 *tiles, int ntiles, int *next,
                     cudaStream_t st, const EnsInteg *mi = nullptr);
// the FP32 pair path's row-profile wind of one component (SWM_CMP_ZONAL or
// SWM_CMP_MERID; null when the wind is not a row profile) and the context's
// (hi, lo) cell-area pairs (3 x ny), for the ensemble's monitored steps
int fused_monitor_inputs(swm_gpu_ctx *c, int comp, float **wind_rows, const float2 **area_pairs);
bool march_std_params(const P32 &p);
// the context's fused path rewrites its forcing fields every step (streams
// other than the nonlinear wind stress, or the mean-state terms)
bool fused_dynamic_forcing(const swm_gpu_ctx *c);
int march_prefetch_level(size_t points, bool integ);
// level 3 (the row ring) serves basins at least this wide; narrower strips
// wrap around the periodic boundary more than once
constexpr int RING_MIN_NX = 32;
// SWM_GPU_EDEVICE when a step kernel's warp gave up waiting for its row
// copies since the library was loaded (reads a device counter; synchronises)
int march_ring_check();
// more bytes than the device's L2 holds
bool exceeds_l2(double bytes);

}  // namespace swm
