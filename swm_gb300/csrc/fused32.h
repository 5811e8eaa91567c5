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

struct P32 {
  int nx, ny, nl, mix, qbf, barotropic, has_F, impl_uniform, gsq_uniform, wind_x, wind_y, wind_rows, has_mode;
  float dt, G, minD, lbc, q1, ts_rho, Ah, bih;
  float ab0, ab1, ab2;
  float impl_s[3], dp_s[3], gsq_s[2];
  const uint16_t *mask16;
  const float *dp[3];
  const float *He, *rows, *Hu, *Hv;
  const float *impl[3], *gsq[2];
  const float *Fx, *Fy, *Fe;
  const float *wx, *wy;
  const float *uh0, *ul0, *vh0, *vl0, *eh0, *el0;
  float *uh1, *ul1, *vh1, *vl1, *eh1, *el1;
  const float *Gu1, *Gu2, *Gv1, *Gv2, *Ge1, *Ge2;
  float *Gu3, *Gv3, *Ge3;
};

// candidate rows per warp strip of the step kernel
constexpr int MARCH_NROWS = 4;
constexpr int MARCH_ROWS[MARCH_NROWS] = {8, 16, 24, 32};

std::vector<double> fp32c_rows(const swm_gpu_ctx *c);
void make_p32(const swm_gpu_ctx *c, int64_t itt, P32 &p);
void march_launch(swm_gpu_ctx *c, const P32 &p);
int march_tile_cols(int mix);          // columns a warp strip updates
int march_rows_override();             // SWM_GB300_MARCH_S, 0 when unset
std::vector<int> march_row_candidates(int mix, int nx, int ny);
int march_pick_rows(cudaStream_t st, int reps, const std::vector<int> &cands, const std::function<void(int)> &launch,
                    int *best);
int march_autotune(swm_gpu_ctx *c, const P32 &p);
void fused_indices(const swm_gpu_ctx *c, int *n0, int *g0);
void fused_set_indices(swm_gpu_ctx *c, int n0, int g0);
void fused_pair_level(const swm_gpu_ctx *c, const float *out[6]);
void fused_static(const swm_gpu_ctx *c, const float **He, const uint16_t **mask16, const float **Fe);
// one launch of the ensemble step: tiles {member, strip << 16 | row group}
int march_ens_launch(int mix, int rows, const P32 *tab, const int2 *tiles, int ntiles, int *next,
                     cudaStream_t st);

}  // namespace swm
