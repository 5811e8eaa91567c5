// march.cu -- FP32 fused SWM step, register-resident row marching.
//
// Each warp owns a strip of 32 columns (lane = column) and S output rows.  It
// walks up the strip one row per iteration, keeping the last rows of every
// intermediate field in registers; x-neighbours come from warp shuffles, so
// the kernel needs no shared memory and no block barrier (the row-ring
// instances, PF = 3, stage their input rows in shared memory).  When row J has
// been loaded, the stress tensor and fluxes needed by row J-2 are complete
// and row J-2 is updated (the biharmonic operator needs two rows of
// look-ahead).  The outer HALO lanes of a strip are recomputed by the
// neighbouring strip, so a strip updates 32 - 2*HALO columns.
//
// Precision: tendencies in binary32; first differences of prognostic fields
// from the (hi, lo) pairs; mass fluxes split into an exact static-depth
// product and the small free-surface product; compensated Adams-Bashforth
// update with the implicit damping applied as x - x*dt*gamma/(1+dt*gamma), so
// the small damping rate keeps its binary32 relative precision (1 + dt*gamma
// itself would lose it).
//
// Formulas: swm_nonlinear_timestep_module.f90:182-449 (diagnostics and
// tendencies), swm_lateralmixing_module.f90:66-240 (stress tensor),
// time_integration_module.f90:74-112 (Adams-Bashforth).
#include <cmath>
#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include <vector>
#include "fused32.h"

// columns per lane of the step kernels (2: march_strip2, packed FP32x2
// arithmetic on 64-column strips; 1: march_strip, 32-column strips), the
// minimum resident blocks per SM asked of the register allocator, and the
// unroll factor of the row loop (tuning knobs, set with -D)
#ifndef MARCH_COLS
#define MARCH_COLS 1
#endif
#ifndef MARCH_MINB
#define MARCH_MINB (MARCH_COLS == 2 ? 2 : 4)
#endif
// integrals formed by the step kernel: 1 = (hi, lo) pair sums of exact
// products; 0 = binary32 sums per lane (a lane holds at most S + 4 rows),
// FP64 across lanes
#ifndef MARCH_INTEG_PAIRS
#define MARCH_INTEG_PAIRS 1
#endif
// 1: the row's cell areas are loaded at the start of the row update
#ifndef MARCH_INTEG_HOIST
#define MARCH_INTEG_HOIST 1
#endif


namespace swm {

constexpr unsigned FULL = 0xffffffffu;
__device__ __forceinline__ float shl(float x) { return __shfl_up_sync(FULL, x, 1); }    // lane - 1
__device__ __forceinline__ float shr(float x) { return __shfl_down_sync(FULL, x, 1); }  // lane + 1

__device__ __forceinline__ int wrapm(int g, int n) {
  g = g < 0 ? g + n : g;
  return g >= n ? g - n : g;
}
__device__ __forceinline__ float rcnt(int c) { return c <= 1 ? 1.f : (c == 2 ? 0.5f : (c == 3 ? 0.33333334f : 0.25f)); }

// ---- row ring (march_strip's PF = 3) ----------------------------------------
//
// Each warp stages the rows it is about to read in a ring of RING slots of
// shared memory, filled by bulk asynchronous copies (cp.async.bulk, the TMA
// engine) and tracked by one mbarrier per slot, so that the compute lanes
// issue no global loads for the state, depth, mask and increments: a slot
// holds, for one input row J, the 32 columns of the warp of the seven state
// and depth fields and of the mask, and the six increments of output row
// J - 2.  A field's row segment is copied as the 16-byte aligned span that
// covers it (bulk copies move whole 16-byte words), in at most two pieces:
// the columns inside [0, nx) and the columns that wrap around the periodic
// boundary; the second piece is placed right after the first.  Allocations
// of the fields leave 16 bytes after their last element, so an aligned span
// never leaves its allocation.  Lanes 0..27 each issue one copy, field
// (lane >> 1), piece (lane & 1).
constexpr int RING = 4;                                // rows in flight per warp
constexpr int RING_FB = 192;                           // one float field (at most 44 floats used)
constexpr int RING_MB = 128;                           // the mask (at most 60 uint16 used)
constexpr int RING_NF = 13;                            // float fields per slot
constexpr int RING_SLOT = RING_NF * RING_FB + RING_MB;  // bytes of one slot
constexpr int RING_WARP = RING * RING_SLOT;            // bytes of one warp's ring
constexpr unsigned long long RING_WAIT_NS = 1000000000ull;  // a row that has not arrived after 1 s

struct RingW {
  const float *ptr;  // the warp's ring
  uint32_t slots;    // its shared-window address
  uint32_t bars;     // and that of its RING mbarriers
  uint32_t phase;    // parity bit of each slot's next phase
};


__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// every lane waits for the phase; false (the same on every lane) when the
// phase has not completed within RING_WAIT_NS
__device__ __forceinline__ bool mbar_wait_warp(uint32_t bar, uint32_t parity) {
  bool done = mbar_try(bar, parity);
  if (__all_sync(FULL, done)) return true;
  const unsigned long long t0 = globaltimer_ns();
  for (;;) {
    if (!done) done = mbar_try(bar, parity);
    if (__all_sync(FULL, done)) return true;
    if (__any_sync(FULL, globaltimer_ns() - t0 > RING_WAIT_NS)) return false;
  }
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
// warps whose row copies did not arrive in time (the step kernels' results
// are then wrong; the host reports it)
__device__ unsigned g_ring_timeouts;

// the ring of warp w of the block and its mbarriers, initialised (every
// lane of the warp calls it)
__device__ __forceinline__ RingW ring_setup(unsigned char *ring, unsigned long long *bars, int w, int lane) {
  RingW r;
  r.ptr = reinterpret_cast<const float *>(ring + (size_t)w * RING_WARP);
  r.slots = smem_addr(ring + (size_t)w * RING_WARP);
  r.bars = smem_addr(bars + w * RING);
  r.phase = 0;
  if (lane == 0) {
    for (int k = 0; k < RING; k++) mbar_init(r.bars + 8u * k, 1);
    mbar_fence_init();
  }
  __syncwarp();
  return r;
}

// mask word: bits 0-3 own (H, u, v, eta), 4-7 column i-1, 8-11 column i+1
#define MH(m) ((m) & 1)
#define MU_(m) (((m) >> 1) & 1)
#define MV_(m) (((m) >> 2) & 1)
#define ME(m) (((m) >> 3) & 1)
#define LV(m) (((m) >> 6) & 1)
#define LE(m) (((m) >> 7) & 1)

// (hi + lo + inc) * (1 - dp) as a new (hi, lo) pair.  Both roundings are
// recovered by Fast2Sum (Dekker 1971), which is exact when the larger operand
// comes first: for s - c always (c = s dp, 0 <= dp < 1); for hi + inc while
// the step's increment is below the state, which fails only where the state
// passes through zero, and there the error left is a rounding of the
// increment, far below the pair's precision relative to the field.
__device__ __forceinline__ void comp_damp(float hi, float lo, float inc, float dp, float &nh, float &nl) {
  const float s = hi + inc;
  float e = (inc - (s - hi)) + lo;
  const float c = s * dp;
  const float t = s - c;
  const float e2 = (s - t) - c;
  e = e + e2 - e * dp;
  nh = t + e;
  nl = e - (nh - t);
}

// One warp updates rows ry0 .. ry0+S-1 of strip bx (columns bx*TI ..
// bx*TI+TI-1) of the basin p describes.  INTEG: each updating lane also adds
// the new state of its ocean points, times the cell area of the point's row
// (area: 3 x ny (hi, lo) pairs, u, v, eta rows), into acc[4]: eta, eta^2,
// u^2, v^2.
// PF: each iteration also asks L2 (prefetch.global.L2, no registers) for the
// next output row's increments (PF >= 1), which it would otherwise load in
// the iteration that uses them, and for the input rows two ahead (PF = 2),
// so that rows not in L2 do not wait on DRAM (march_prefetch_level).
// PF = 3: the rows come through the warp's row ring rw instead (bulk copies
// RING - 1 rows ahead; needs nx >= RING_MIN_NX).  Returns false when a row
// did not arrive in time (the warp's copies still in flight are waited for,
// within the same limit, before it returns).
template <int MIX, bool INTEG = false, bool STD = false, int PF = 0>
__device__ __forceinline__ bool march_strip(const P32 &p, const int bx, const int ry0, const int lane, const int S,
                                            const float2 *area = nullptr, F2 *acc = nullptr,
                                            RingW *rw = nullptr) {
  constexpr bool RG = PF == 3;
  constexpr int H = MIX == 2 ? 2 : 1;
  constexpr int TI = 32 - 2 * H;
  const int nx = p.nx, ny = p.ny;
  const int gx = bx * TI - H + lane;
  const int gi = ((gx % nx) + nx) % nx;  // periodic in i; narrow basins stay in bounds
  // STD: the configuration flags of march_std() hold, as compile-time constants
  const bool nl = STD || p.nl, has_mode = STD || p.has_mode, qbf = !STD && p.qbf, has_F = !STD && p.has_F;
  const bool impl_uniform = STD || p.impl_uniform, wind_rows = STD || p.wind_rows;
  const bool store_lane = lane >= H && lane < 32 - H && gx < nx;
  const float q1 = p.q1, G = p.G;

  // sliding windows, index a = row J - a
  float uh[4] = {}, ul[4] = {}, vh[4] = {}, vl[4] = {}, eh[4] = {}, el[4] = {}, he[4] = {};
  unsigned m[4] = {};
  float pll1[2] = {}, plt1[2] = {}, lu1[2] = {}, lv1[2] = {}, pll2[2] = {}, plt2[2] = {};
  float muh[4] = {}, mul[4] = {}, mvh[3] = {}, mvl[3] = {}, pot[3] = {}, ke[3] = {};
  int off[3] = {};            // row offsets nx * j of rows J, J-1, J-2

  int J = ry0 - 3;
  const int J0 = J;
  const int jend = min(ry0 + S, ny) + 2;
  int noff = nx * wrapm(J, ny);
  unsigned n_m = 0;
  float n_uh = 0.f, n_ul = 0.f, n_vh = 0.f, n_vl = 0.f, n_eh = 0.f, n_el = 0.f, n_he = 0.f;
  if (!RG) {
    n_m = p.mask16[gi + noff];
    n_uh = p.uh0[gi + noff]; n_ul = p.ul0[gi + noff]; n_vh = p.vh0[gi + noff]; n_vl = p.vl0[gi + noff];
    n_eh = p.eh0[gi + noff]; n_el = p.el0[gi + noff]; n_he = p.He[gi + noff];
  }

  // ---- row ring (PF = 3) ----
  // the warp's columns gx0 .. gx0+31: piece 0 [am, am+wm) inside the basin,
  // piece 1 [aw, aw+ww) the columns that wrap around
  const int gx0 = bx * TI - H;
  const int am = max(gx0, 0), wm = min(gx0 + 32, nx) - am;
  const int aw = gx0 < 0 ? gx0 + nx : 0, ww = gx0 < 0 ? -gx0 : max(gx0 + 32 - nx, 0);
  const bool inw = gx < 0 || gx >= nx;
  const int lofs = gi - (inw ? aw : am);  // the lane's column within its piece
  // element index of the lane's column in a field's slot region, for the
  // row at offset r and an alignment of al + 1 elements
  auto ridx = [&](int r, int al) {
    const int s0 = (r + am) & al;
    return inw ? ((s0 + wm + al) & ~al) + ((r + aw) & al) + lofs : s0 + lofs;
  };
  // the lane's copy: field fi (0-6 uh ul vh vl eh el He of row J, 7-12
  // Ge1 Ge2 Gu1 Gu2 Gv1 Gv2 of row J-2, 13 the mask of row J), piece pc
  const int fi = lane >> 1, pc = lane & 1;
  const int pa = pc ? aw : am, pw = pc ? ww : wm;
  const int fes = fi == 13 ? 2 : 4, fal = fi == 13 ? 7 : 3;
  const char *fsrc = nullptr;
  if (RG) {
    const void *f = nullptr;
    switch (fi) {
      case 0: f = p.uh0; break;
      case 1: f = p.ul0; break;
      case 2: f = p.vh0; break;
      case 3: f = p.vl0; break;
      case 4: f = p.eh0; break;
      case 5: f = p.el0; break;
      case 6: f = p.He; break;
      case 7: f = p.Ge1; break;
      case 8: f = p.Ge2; break;
      case 9: f = p.Gu1; break;
      case 10: f = p.Gu2; break;
      case 11: f = p.Gv1; break;
      case 12: f = p.Gv2; break;
      case 13: f = p.mask16; break;
      default: break;
    }
    fsrc = static_cast<const char *>(f);
  }
  // copies of input row Jr and of the increments of output row Jr - 2 into
  // the slot of Jr
  auto issue = [&](int Jr) {
    const int s = (Jr - J0) & (RING - 1);
    const uint32_t bar = rw->bars + 8u * s;
    const int o = Jr - 2;
    const bool incr = fi >= 7 && fi <= 12;
    const bool act = fsrc != nullptr && pw > 0 && (!incr || (o >= ry0 && o < ry0 + S && o < ny));
    uint32_t bytes = 0, dst = 0;
    const char *src = nullptr;
    if (act) {
      const int r = nx * (incr ? o : wrapm(Jr, ny));
      const int s0 = (r + pa) & fal;
      bytes = (uint32_t)(((s0 + pw + fal) & ~fal) * fes);
      const int before = pc ? (((r + am) & fal) + wm + fal) & ~fal : 0;  // elements of piece 0
      dst = rw->slots + (uint32_t)(s * RING_SLOT + (fi == 13 ? RING_NF * RING_FB : fi * RING_FB) + before * fes);
      src = fsrc + (size_t)(r + pa - s0) * fes;
    }
    const uint32_t tx = __reduce_add_sync(FULL, bytes);
    if (lane == 0) mbar_expect_tx(bar, tx);
    __syncwarp();
    if (act) bulk_g2s(dst, src, bytes, bar);
  };
  const float *rs = nullptr;  // the slot of the current row, as floats
  if (RG)
    for (int k = 0; k < RING - 1; k++)
      if (J0 + k < jend) issue(J0 + k);

  // one iteration; FAST: every cell of the warp's 4-row window is ocean on
  // all four grids, so every mask test is compile-time true
  auto body = [&](auto fast_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
#define XH(m_) (FAST ? 1u : MH(m_))
#define XU(m_) (FAST ? 1u : MU_(m_))
#define XV(m_) (FAST ? 1u : MV_(m_))
#define XE(m_) (FAST ? 1u : ME(m_))
#define XLV(m_) (FAST ? 1u : LV(m_))
#define XLE(m_) (FAST ? 1u : LE(m_))
#define W2(a_, b_) (FAST ? 0.5f : rcnt((a_) + (b_)))
#define W4(a_, b_, c_, d_) (FAST ? 0.25f : rcnt((a_) + (b_) + (c_) + (d_)))
#define HALF2(a_, b_) (FAST ? 0.5f : ((a_) + (b_) > 1 ? 0.5f : 1.f))
    auto dval = [&](int a) { return nl ? (XE(m[a]) ? he[a] + eh[a] : 1.f) : he[a]; };
    const float4 *rec = p.rec + (size_t)wrapm(J, ny) * REC_N;  // factors of rows J, J-1, J-2
    // all record loads issued first, so their latency overlaps the fluxes
    const float4 fa = rec[REC_A], fb = rec[REC_B], fc = rec[REC_C], fd = rec[REC_D], fe = rec[REC_E],
                 ff = rec[REC_F];
    const float fh = reinterpret_cast<const float *>(rec + REC_G)[0];
    const int o = J - 2;
    const bool upd = o >= ry0 && o < ry0 + S && o < ny && store_lane;
    const int ko = gi + off[2];
    float g1e = 0, g2e = 0, g1u = 0, g2u = 0, g1v = 0, g2v = 0;
    // row-profile wind of row o, loaded with the increments (not in the
    // monitored instances, whose sums leave no register for it)
    float wxo = 0.f, wyo = 0.f;
    if (upd) {
      if (RG) {
        constexpr int FW = RING_FB / 4;
        const float *g = rs + ridx(off[2], 3);
        g1e = g[7 * FW]; g2e = g[8 * FW]; g1u = g[9 * FW]; g2u = g[10 * FW]; g1v = g[11 * FW]; g2v = g[12 * FW];
      } else {
        g1e = p.Ge1[ko]; g2e = p.Ge2[ko]; g1u = p.Gu1[ko]; g2u = p.Gu2[ko]; g1v = p.Gv1[ko]; g2v = p.Gv2[ko];
      }
      if (!INTEG && wind_rows) {
        if (p.wind_x) wxo = p.wx[o];
        if (p.wind_y) wyo = p.wy[o];
      }
    }

    // ---- row J: mass fluxes and PV; row J-1: kinetic energy ----------
    const float d0 = dval(0), d1 = dval(1), d2 = dval(2), d3 = dval(3);
    const float he_l = shl(he[0]), eh_l = shl(eh[0]);
    const float dl0 = shl(d0), dl1 = shl(d1), dl2 = shl(d2);
    const float vh0_l = shl(vh[0]), vl0_l = shl(vl[0]);
    const float uh1_r = shr(uh[1]), ul1_r = shr(ul[1]);
    {
      const unsigned mm = m[0];
      float a_h = 0.f, a_l = 0.f;
      if (XU(mm)) {
        unsigned a = XE(mm), b = XLE(mm);
        float w = W2(a, b);
        float hs = ((a ? he[0] : 0.f) + (b ? he_l : 0.f)) * w;
        float es = nl ? ((a ? eh[0] : 0.f) + (b ? eh_l : 0.f)) * w : 0.f;
        a_h = hs * uh[0];
        a_l = fmaf(hs, uh[0], -a_h) + fmaf(hs, ul[0], es * uh[0]);
      }
      muh[0] = a_h; mul[0] = a_l;
      float b_h = 0.f, b_l = 0.f;
      if (XV(mm)) {
        unsigned a = XE(mm), b = XE(m[1]);
        float w = W2(a, b);
        float hs = ((a ? he[0] : 0.f) + (b ? he[1] : 0.f)) * w;
        float es = nl ? ((a ? eh[0] : 0.f) + (b ? eh[1] : 0.f)) * w : 0.f;
        b_h = hs * vh[0];
        b_l = fmaf(hs, vh[0], -b_h) + fmaf(hs, vl[0], es * vh[0]);
      }
      mvh[0] = b_h; mvl[0] = b_l;
      float pv = 0.f;
      if (has_mode) {
        float zeta = 0.f;
        if (nl) {
          float bc = XH(mm) ? 1.f : p.lbc;
          float dvdx = (XLV(mm) + XV(mm) == 0) ? 0.f : bc * fa.x * ((vh[0] - vh0_l) + (vl[0] - vl0_l));
          float dudy = (XU(mm) + XU(m[1]) == 0)
                           ? 0.f
                           : bc * q1 * (fa.y * ((uh[0] - uh[1]) + (ul[0] - ul[1])) + fa.z * uh[1]);
          zeta = dvdx - dudy * fa.w;
        }
        unsigned a = XE(mm), b = XLE(m[1]), c = XLE(mm), d = XE(m[1]);
        float dh = ((a ? d0 : 0.f) + (b ? dl1 : 0.f) + (c ? dl0 : 0.f) + (d ? d1 : 0.f)) * W4(a, b, c, d);
        pv = __fdividef(fh + zeta, fmaxf(dh, 2.220446e-16f));
      }
      pot[0] = pv;
      float k1 = 0.f;
      if (nl && XE(m[1])) {
        float a = 0.5f * (uh1_r * uh1_r) + 0.5f * (uh[1] * uh[1]);
        float c = 0.5f * (vh[0] * vh[0]) + 0.5f * (vh[1] * vh[1]);
        k1 = (a + c) * 0.5f;
      }
      ke[0] = k1;
    }

    // ---- lateral stress: pll2 at row J-2, plt2 at row J-1 -------------
    if (MIX == 2) {
      {  // first pass, unit thickness, Ah = 1: pll1 at J-1, plt1 at J
        const unsigned m1 = m[1], m0 = m[0];
        float pl = 0.f, pt = 0.f;
        if (XE(m1)) {
          unsigned ov = XV(m1), ovp = XV(m0);
          float tE = fb.x * HALF2(ov, ovp);
          float du = (uh1_r - uh[1]) + (ul1_r - ul[1]);
          float dv = (vh[0] - vh[1]) + (vl[0] - vl[1]);
          pl = fb.y * du + q1 * dv + tE * ((ovp ? vh[0] : 0.f) + (ov ? vh[1] : 0.f));
        }
        if (XH(m0)) {
          unsigned ou = XU(m0), oum = XU(m1);
          float tH = fb.z * HALF2(ou, oum);
          float dv = (vh[0] - vh0_l) + (vl[0] - vl0_l);
          float du = (uh[0] - uh[1]) + (ul[0] - ul[1]);
          pt = fb.w * dv - q1 * du - tH * ((ou ? uh[0] : 0.f) + (oum ? uh[1] : 0.f));
        }
        pll1[0] = pl;
        plt1[0] = pt;
      }
      {  // lu1, lv1 at row J-1
        const float pll1_l = shl(pll1[0]), plt1_r = shr(plt1[1]);
        const unsigned m1 = m[1];
        float a = 0.f, b = 0.f;
        if (XU(m1)) {
          float t2 = 2.f * fc.x * HALF2(XH(m1), XH(m[0]));
          a = -fc.y * (pll1[0] - pll1_l) + q1 * (plt1[1] - plt1[0]) + t2 * (plt1[0] + plt1[1]);
        }
        if (XV(m1)) {
          float t2 = 2.f * fc.z * HALF2(XE(m1), XE(m[2]));
          b = -fc.w * (plt1_r - plt1[1]) + q1 * (pll1[0] - pll1[1]) - t2 * (pll1[0] + pll1[1]);
        }
        lu1[0] = a;
        lv1[0] = b;
      }
      {  // second pass, thickness weighted, Ah = -bih
        const float lu1_r = shr(lu1[1]), lv1_l = shl(lv1[0]);
        const unsigned m2 = m[2], m1 = m[1];
        float pl = 0.f, pt = 0.f;
        if (XE(m2)) {
          unsigned ov = XV(m2), ovp = XV(m1);
          float tE = fd.x * HALF2(ov, ovp);
          float s = fd.y * (lu1_r - lu1[1]) + q1 * (lv1[0] - lv1[1]) +
                    tE * ((ovp ? lv1[0] : 0.f) + (ov ? lv1[1] : 0.f));
          pl = -p.bih * d2 * s;
        }
        if (XH(m1)) {
          unsigned ou = XU(m1), oum = XU(m2);
          float tH = fd.z * HALF2(ou, oum);
          float s = fd.w * (lv1[0] - lv1_l) - q1 * (lu1[0] - lu1[1]) -
                    tH * ((ou ? lu1[0] : 0.f) + (oum ? lu1[1] : 0.f));
          unsigned a = XE(m1), b = XLE(m2), c = XLE(m1), d = XE(m2);
          float dh = ((a ? d1 : 0.f) + (b ? dl2 : 0.f) + (c ? dl1 : 0.f) + (d ? d2 : 0.f)) * W4(a, b, c, d);
          pt = -p.bih * dh * s;
        }
        pll2[0] = pl;
        plt2[0] = pt;
      }
    } else if (MIX == 1) {
      const float uh2_r = shr(uh[2]), ul2_r = shr(ul[2]);
      const float vh1_l = shl(vh[1]), vl1_l = shl(vl[1]);
      const unsigned m2 = m[2], m1 = m[1];
      float pl = 0.f, pt = 0.f;
      if (XE(m2)) {
        unsigned ov = XV(m2), ovp = XV(m1);
        float tE = fd.x * HALF2(ov, ovp);
        float du = (uh2_r - uh[2]) + (ul2_r - ul[2]);
        float dv = (vh[1] - vh[2]) + (vl[1] - vl[2]);
        float s = fd.y * du + q1 * dv + tE * ((ovp ? vh[1] : 0.f) + (ov ? vh[2] : 0.f));
        pl = p.Ah * d2 * s;
      }
      if (XH(m1)) {
        unsigned ou = XU(m1), oum = XU(m2);
        float tH = fd.z * HALF2(ou, oum);
        float dv = (vh[1] - vh1_l) + (vl[1] - vl1_l);
        float du = (uh[1] - uh[2]) + (ul[1] - ul[2]);
        float s = fd.w * dv - q1 * du - tH * ((ou ? uh[1] : 0.f) + (oum ? uh[2] : 0.f));
        unsigned a = XE(m1), b = XLE(m2), c = XLE(m1), d = XE(m2);
        float dh = ((a ? d1 : 0.f) + (b ? dl2 : 0.f) + (c ? dl1 : 0.f) + (d ? d2 : 0.f)) * W4(a, b, c, d);
        pt = p.Ah * dh * s;
      }
      pll2[0] = pl;
      plt2[0] = pt;
    }

    // ---- tendencies and compensated update of row o = J-2 ------------
    // every lane takes part in the shuffles; updating lanes use the values
    // the PV fluxes take the whole mass flux, hi + lo: lo carries the
    // free-surface part eta * u, which is not a rounding-level correction
    const float mvs1 = mvh[1] + mvl[1], mvs2 = mvh[2] + mvl[2];
    const float mus2 = muh[2] + mul[2], mus3 = muh[3] + mul[3];
    const float muh2_r = shr(muh[2]), mul2_r = shr(mul[2]), mus3_r = shr(mus3);
    const float mvs2_l = shl(mvs2), mvs1_l = shl(mvs1);
    const float eh2_l = shl(eh[2]), el2_l = shl(el[2]), ke1_l = shl(ke[1]);
    const float pot2_r = shr(pot[2]);
    const float vh2_l = shl(vh[2]), vh1_lo = shl(vh[1]);
    const float uh2_r = shr(uh[2]), uh3_r = shr(uh[3]);
    const float pll2_l = shl(pll2[0]), plt2_r = shr(plt2[1]);
    if (upd) {
      const unsigned mm = m[2];
      float ge = 0.f, gu = 0.f, gv = 0.f;
      // INTEG: the row's cell areas, loaded here so that their latency
      // overlaps the tendencies
      float2 aru, arv, are;
      if (INTEG && MARCH_INTEG_HOIST) {
        aru = area[o];
        arv = area[ny + o];
        are = area[2 * ny + o];
      }
      if (XE(mm)) {
        // cos_{o+1} MV_{o+1} - cos_o MV_o as cos_{o+1} (MV_{o+1} - MV_o) +
        // (cos_{o+1} - cos_o) MV_o; the second product takes the whole MV_o,
        // hi + lo, because lo holds the free-surface part eta * v
        float dmv = fe.x * ((mvh[1] - mvh[2]) + (mvl[1] - mvl[2])) + fe.y * mvs2;
        ge = -((muh2_r - muh[2]) + (mul2_r - mul[2])) * fe.z - dmv * fe.w;
        if (has_F) ge += p.Fe[ko];
      }
      if (XU(mm)) {
        float pv = 0.5f * (pot[1] + pot[2]);
        float mv = 0.25f * ((mvs1 + mvs2_l) + (mvs1_l + mvs2));
        float dE = G * ((eh[2] - eh2_l) + (el[2] - el2_l)) + (ke[1] - ke1_l);
        float g = pv * mv - dE * ff.x;
        unsigned a = XE(mm), b = XLE(mm);
        float du = ((a ? d2 : 0.f) + (b ? dl2 : 0.f)) * W2(a, b);
        if (qbf) {
          float vb = 0.25f * ((vh[1] + vh2_l) + (vh1_lo + vh[2]));
          float gs = p.gsq_uniform ? p.gsq_s[0] : p.gsq[0][ko];
          float f = gs * sqrtf(uh[2] * uh[2] + vb * vb) * uh[2];
          if (p.barotropic) f = __fdividef(f, p.Hu[ko]);
          g -= f;
        }
        if (MIX) {
          float t2 = 2.f * ff.y * HALF2(XH(mm), XH(m[1]));
          float lat = -ff.x * (pll2[0] - pll2_l) + q1 * (plt2[1] - plt2[0]) + t2 * (plt2[0] + plt2[1]);
          g += __fdividef(lat, du);
        }
        if (has_F) g += p.Fx[ko];
        if (p.wind_x) g += __fdividef(p.ts_rho * (wind_rows ? (INTEG ? p.wx[o] : wxo) : p.wx[ko]), nl ? du : 1.f);
        gu = g;
      }
      if (XV(mm)) {
        float pv = 0.5f * (pot2_r + pot[2]);
        float mu = 0.25f * (((muh2_r + mul2_r) + mus3) + (mus2 + mus3_r));
        float dE = G * ((eh[2] - eh[3]) + (el[2] - el[3])) + (ke[1] - ke[2]);
        float g = -pv * mu - dE * q1;
        unsigned a = XE(mm), b = XE(m[3]);
        float dv = ((a ? d2 : 0.f) + (b ? d3 : 0.f)) * W2(a, b);
        if (qbf) {
          float ub = 0.25f * ((uh2_r + uh[3]) + (uh[2] + uh3_r));
          float gs = p.gsq_uniform ? p.gsq_s[1] : p.gsq[1][ko];
          float f = gs * sqrtf(vh[2] * vh[2] + ub * ub) * vh[2];
          if (p.barotropic) f = __fdividef(f, p.Hv[ko]);
          g -= f;
        }
        if (MIX) {
          float t2 = 2.f * ff.z * HALF2(XE(mm), XE(m[3]));
          float lat = -ff.w * (plt2_r - plt2[1]) + q1 * (pll2[0] - pll2[1]) - t2 * (pll2[0] + pll2[1]);
          g += __fdividef(lat, dv);
        }
        if (has_F) g += p.Fy[ko];
        if (p.wind_y) g += __fdividef(p.ts_rho * (wind_rows ? (INTEG ? p.wy[o] : wyo) : p.wy[ko]), nl ? dv : 1.f);
        gv = g;
      }
      p.Ge3[ko] = ge;
      p.Gu3[ko] = gu;
      p.Gv3[ko] = gv;
      float dpu, dpv, dpe;
      if (impl_uniform) {
        dpu = p.dp_s[0]; dpv = p.dp_s[1]; dpe = p.dp_s[2];
      } else {
        dpu = p.dp[0][ko]; dpv = p.dp[1][ko]; dpe = p.dp[2][ko];
      }
      float ince = p.dt * (p.ab0 * g1e + p.ab1 * g2e + p.ab2 * ge);
      float incu = p.dt * (p.ab0 * g1u + p.ab1 * g2u + p.ab2 * gu);
      float incv = p.dt * (p.ab0 * g1v + p.ab1 * g2v + p.ab2 * gv);
      float nh, nlo;
      comp_damp(eh[2], el[2], ince, dpe, nh, nlo);
      if (nl) {
        float lim = p.minD - he[2];
        if (nh < lim) { nh = lim; nlo = 0.f; }
      }
      p.eh1[ko] = nh; p.el1[ko] = nlo;
      if (INTEG && !MARCH_INTEG_HOIST) {
        aru = area[o];
        arv = area[ny + o];
        are = area[2 * ny + o];
      }
      F2 sq;
      if (INTEG && XE(mm)) {
        if (MARCH_INTEG_PAIRS) {
          F2 x;
          x.h = nh;
          x.l = nlo;
          acc[0].add_prod(are, x);
          sq_pair(nh, nlo, sq.h, sq.l);
          acc[1].add_prod(are, sq);
        } else {
          const float x = nh + nlo;
          acc[0].h = fmaf(are.x, x, acc[0].h);
          acc[1].h = fmaf(are.x, x * x, acc[1].h);
        }
      }
      comp_damp(uh[2], ul[2], incu, dpu, nh, nlo);
      p.uh1[ko] = nh; p.ul1[ko] = nlo;
      if (INTEG && XU(mm)) {
        if (MARCH_INTEG_PAIRS) {
          sq_pair(nh, nlo, sq.h, sq.l);
          acc[2].add_prod(aru, sq);
        } else {
          acc[2].h = fmaf(aru.x, nh * nh, acc[2].h);
        }
      }
      comp_damp(vh[2], vl[2], incv, dpv, nh, nlo);
      p.vh1[ko] = nh; p.vl1[ko] = nlo;
      if (INTEG && XV(mm)) {
        if (MARCH_INTEG_PAIRS) {
          sq_pair(nh, nlo, sq.h, sq.l);
          acc[3].add_prod(arv, sq);
        } else {
          acc[3].h = fmaf(arv.x, nh * nh, acc[3].h);
        }
      }
    }
#undef XH
#undef XU
#undef XV
#undef XE
#undef XLV
#undef XLE
#undef W2
#undef W4
#undef HALF2
  };

#ifdef MARCH_UNROLL
#define MARCH_PRAGMA_(x) _Pragma(#x)
#define MARCH_PRAGMA(x) MARCH_PRAGMA_(x)
  MARCH_PRAGMA(unroll MARCH_UNROLL)
#endif
  for (; J < jend; J++) {
#pragma unroll
    for (int a = 3; a > 0; a--) {
      uh[a] = uh[a - 1]; ul[a] = ul[a - 1]; vh[a] = vh[a - 1]; vl[a] = vl[a - 1];
      eh[a] = eh[a - 1]; el[a] = el[a - 1]; he[a] = he[a - 1]; m[a] = m[a - 1];
      muh[a] = muh[a - 1]; mul[a] = mul[a - 1];
    }
#pragma unroll
    for (int a = 2; a > 0; a--) {
      mvh[a] = mvh[a - 1]; mvl[a] = mvl[a - 1]; pot[a] = pot[a - 1]; ke[a] = ke[a - 1];
      off[a] = off[a - 1];
    }
    pll1[1] = pll1[0]; plt1[1] = plt1[0]; lu1[1] = lu1[0]; lv1[1] = lv1[0];
    pll2[1] = pll2[0]; plt2[1] = plt2[0];
    if (RG) {
      // the slot of row J + RING - 1 is the one row J - 1 used: every lane
      // has read it (warp barrier) before the copies overwrite it
      __syncwarp();
      if (J + RING - 1 < jend) issue(J + RING - 1);
      const int sl = (J - J0) & (RING - 1);
      if (!mbar_wait_warp(rw->bars + 8u * sl, (rw->phase >> sl) & 1u)) {
        // the rows issued after this one: wait for their copies (each again
        // within the limit) so that none lands after the warp has left
        for (int k = 1; k < RING && J + k < jend; k++) {
          const int s2 = (J + k - J0) & (RING - 1);
          mbar_wait_warp(rw->bars + 8u * s2, (rw->phase >> s2) & 1u);
        }
        return false;
      }
      rw->phase ^= 1u << sl;
      constexpr int FW = RING_FB / 4;
      rs = rw->ptr + sl * (RING_SLOT / 4);
      const float *f = rs + ridx(noff, 3);
      uh[0] = f[0]; ul[0] = f[FW]; vh[0] = f[2 * FW]; vl[0] = f[3 * FW];
      eh[0] = f[4 * FW]; el[0] = f[5 * FW]; he[0] = f[6 * FW];
      m[0] = reinterpret_cast<const uint16_t *>(rs + RING_NF * FW)[ridx(noff, 7)];
      off[0] = noff;
      if (J + 1 < jend) noff = nx * wrapm(J + 1, ny);
    } else {
      m[0] = n_m; uh[0] = n_uh; ul[0] = n_ul; vh[0] = n_vh; vl[0] = n_vl;
      eh[0] = n_eh; el[0] = n_el; he[0] = n_he;
      off[0] = noff;
      if (J + 1 < jend) {  // prefetch row J+1
        int jw = wrapm(J + 1, ny);
        noff = nx * jw;
        const int kn = gi + noff;
        n_m = p.mask16[kn];
        n_uh = p.uh0[kn]; n_ul = p.ul0[kn]; n_vh = p.vh0[kn]; n_vl = p.vl0[kn];
        n_eh = p.eh0[kn]; n_el = p.el0[kn]; n_he = p.He[kn];
      }
    }
    if (PF == 1 || PF == 2) {
      if (PF == 2 && J + 2 < jend) {  // the input rows two ahead
        const int k2 = gi + nx * wrapm(J + 2, ny);
        prefetch_l2(p.mask16 + k2);
        prefetch_l2(p.uh0 + k2); prefetch_l2(p.ul0 + k2); prefetch_l2(p.vh0 + k2); prefetch_l2(p.vl0 + k2);
        prefetch_l2(p.eh0 + k2); prefetch_l2(p.el0 + k2); prefetch_l2(p.He + k2);
      }
      if (store_lane && J - 1 >= ry0 && J - 1 < ry0 + S && J - 1 < ny) {  // the next output row's increments
        const int k1 = gi + off[1];
        prefetch_l2(p.Ge1 + k1); prefetch_l2(p.Ge2 + k1); prefetch_l2(p.Gu1 + k1);
        prefetch_l2(p.Gu2 + k1); prefetch_l2(p.Gv1 + k1); prefetch_l2(p.Gv2 + k1);
      }
    }
    // rows ry0-3 and ry0-2 only fill the windows: nothing computed from them
    // reaches an output row (the first, ry0, needs first-pass stresses from
    // row ry0-2 on, formed once row ry0-1 is in)
    if (J < ry0 - 1) continue;
    const bool interior = __all_sync(FULL, (m[0] & m[1] & m[2] & m[3] & 0xFFFu) == 0xFFFu);
    if (interior) body(std::true_type{});
    else body(std::false_type{});
  }
  return true;
}

#if MARCH_COLS == 2
#include "march2.cuh"
#define MARCH_STRIP march_strip2
#else
#define MARCH_STRIP march_strip
#endif

// End of a strip block of k_march<MIX, true>: each warp reduces its lanes'
// pair sums (shuffle tree), then thread 0 adds the four warps in order in
// FP64 and stores the block's sums as block b of nb.
__device__ __forceinline__ void march_integrals_block(const MarchInteg &mi, F2 *acc, int b, int nb) {
  __shared__ double red[4][4];
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float h = __shfl_down_sync(FULL, acc[q].h, o), l = __shfl_down_sync(FULL, acc[q].l, o);
      acc[q].add(h, l);
    }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int q = 0; q < 4; q++) red[q][warp] = acc[q].value();
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < 4; q++) mi.partial[(size_t)q * nb + b] = ((red[q][0] + red[q][1]) + red[q][2]) + red[q][3];
}

// The three integrals from nb per-block sums, by one block of 128 threads:
// thread t adds blocks t, t + 128, ... (BATCH loads at a time), then the
// shuffle tree, then the four warps in order.
__device__ __forceinline__ void integrals_from_blocks(const double *partial, int nb, double G, double *out) {
  __shared__ double red[4][4];
  constexpr int BATCH = 8;
  double t[4] = {0., 0., 0., 0.};
  for (int b0 = threadIdx.x; b0 < nb; b0 += BATCH * 128) {
    double v[4][BATCH];
#pragma unroll
    for (int k = 0; k < BATCH; k++) {
      const int b = b0 + k * 128;
#pragma unroll
      for (int q = 0; q < 4; q++) v[q][k] = b < nb ? partial[(size_t)q * nb + b] : 0.;
    }
#pragma unroll
    for (int k = 0; k < BATCH; k++)
#pragma unroll
      for (int q = 0; q < 4; q++) t[q] += v[q][k];
  }
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 4; q++) t[q] += __shfl_down_sync(FULL, t[q], o);
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int q = 0; q < 4; q++) red[q][warp] = t[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double a[4];
#pragma unroll
    for (int q = 0; q < 4; q++) a[q] = ((red[q][0] + red[q][1]) + red[q][2]) + red[q][3];
    out[0] = a[0];
    out[1] = 0.5 * G * a[1];
    out[2] = 0.5 * (a[2] + a[3]);
  }
}

// block 0 of a monitored step: the next step's wind rows, then the previous
// step's integrals
__device__ __forceinline__ void march_monitor_jobs(const MarchInteg &mi, int nb) {
  if (mi.next_rows)
    for (int j = threadIdx.x; j < mi.ny; j += blockDim.x) mi.next_w[j] = (float)mi.next_rows[j];
  if (mi.prev_partial) integrals_from_blocks(mi.prev_partial, nb, mi.G, mi.prev_out);
}

// the last monitored step's integrals (launched after its step kernel, as its
// programmatic dependent)
__global__ void __launch_bounds__(128) k_march_integrals_final(const double *__restrict__ partial, int nb, double G,
                                                                double *out) {
  grid_dep_wait();
  integrals_from_blocks(partial, nb, G, out);
}

void march_integrals_final(const double *partial, int nb, double G, double *out, cudaStream_t st) {
  launch_programmatic(k_march_integrals_final, dim3(1), dim3(128), st, partial, nb, G, out);
}

// Warp w of block b takes tile 4 b + w of `tiles`: {strip, first row << 8 |
// rows} (rows 0: nothing to do).  A block's four tiles are consecutive row
// groups of one strip, so their look-ahead rows overlap and meet in L1.
// INTEG (a monitored step, MarchInteg): block 0 does the side jobs and the
// strip blocks are blockIdx.x - 1; they sum the new state as well.
template <int MIX, bool INTEG, bool STD, int PF>
__global__ void __launch_bounds__(128, MARCH_MINB) k_march(P32 p, const int2 *__restrict__ tiles, MarchInteg mi) {
  const int lane = threadIdx.x & 31;
  int b = blockIdx.x;
  if (INTEG) {
    grid_dep_wait();
    if (b == 0) {
      march_monitor_jobs(mi, gridDim.x - 1);
      return;
    }
    b -= 1;
  }
  const int2 t = tiles[4 * b + (threadIdx.x >> 5)];
  const int S = t.y & 255;
  F2 acc[4];
  __shared__ __align__(128) unsigned char ring[PF == 3 ? 4 * RING_WARP : 16];
  __shared__ unsigned long long rbar[PF == 3 ? 4 * RING : 1];
  if (S > 0) {
    if constexpr (PF == 3) {
      RingW rw = ring_setup(ring, rbar, threadIdx.x >> 5, lane);
      if (!march_strip<MIX, INTEG, STD, PF>(p, t.x, t.y >> 8, lane, S, mi.area, acc, &rw) && lane == 0)
        atomicAdd(&g_ring_timeouts, 1u);
    } else {
      MARCH_STRIP<MIX, INTEG, STD, PF>(p, t.x, t.y >> 8, lane, S, mi.area, acc);
    }
  }
  if (INTEG) {
    grid_dep_trigger();
    march_integrals_block(mi, acc, b, gridDim.x - 1);
  }
}

// Ensemble of basins in one persistent launch: every warp takes tiles from
// the queue until it is empty.  A tile is int4 {member, strip, first row,
// rows}; the member's parameter block is copied into the warp's slice of
// shared memory first.
// INTEG (monitored ensemble steps): each warp also sums the new state of its
// tile's ocean points times the member's cell areas (areas[member], 3 x ny
// (hi, lo) pairs) and writes the tile's four sums, eta, eta^2, u^2 and v^2
// times area, to partial[4 * tile + q]; k_ens_tile_sums adds them per member.
template <int MIX, bool STD, int PF, bool INTEG>
__global__ void __launch_bounds__(128, MARCH_MINB) k_march_ens(const P32 *__restrict__ tab,
                                                               const int4 *__restrict__ tiles, int ntiles,
                                                               int *__restrict__ next,
                                                               const float2 *const *__restrict__ areas,
                                                               double *__restrict__ partial) {
  __shared__ P32 sp[4];
  __shared__ __align__(128) unsigned char ring[PF == 3 ? 4 * RING_WARP : 16];
  __shared__ unsigned long long rbar[PF == 3 ? 4 * RING : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (INTEG) grid_dep_wait();  // monitored steps are launched programmatically
  RingW rw{};
  if (PF == 3) rw = ring_setup(ring, rbar, warp, lane);
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(next, 1);
    t = __shfl_sync(FULL, t, 0);
    if (t >= ntiles) return;
    const int4 d = tiles[t];
    const int *src = reinterpret_cast<const int *>(tab + d.x);
    int *dst = reinterpret_cast<int *>(&sp[warp]);
    for (int k = lane; k < (int)(sizeof(P32) / sizeof(int)); k += 32) dst[k] = src[k];
    __syncwarp();
    if (PF == 3) {
      bool ok;
      if (INTEG) {
        F2 acc[4];
        ok = march_strip<MIX, true, STD, PF>(sp[warp], d.y, d.z, lane, d.w, areas[d.x], acc, &rw);
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const float h = __shfl_down_sync(FULL, acc[q].h, o), l = __shfl_down_sync(FULL, acc[q].l, o);
            acc[q].add(h, l);
          }
        if (lane == 0)
#pragma unroll
          for (int q = 0; q < 4; q++) partial[4 * (size_t)t + q] = acc[q].value();
      } else {
        ok = march_strip<MIX, false, STD, PF>(sp[warp], d.y, d.z, lane, d.w, nullptr, nullptr, &rw);
      }
      if (!ok) {
        if (lane == 0) atomicAdd(&g_ring_timeouts, 1u);
        return;
      }
    } else if (INTEG) {
      F2 acc[4];
      MARCH_STRIP<MIX, true, STD, PF>(sp[warp], d.y, d.z, lane, d.w, areas[d.x], acc);
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const float h = __shfl_down_sync(FULL, acc[q].h, o), l = __shfl_down_sync(FULL, acc[q].l, o);
          acc[q].add(h, l);
        }
      if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; q++) partial[4 * (size_t)t + q] = acc[q].value();
    } else {
      MARCH_STRIP<MIX, false, STD, PF>(sp[warp], d.y, d.z, lane, d.w);
    }
    __syncwarp();
  }
}

// per-row factors for the FP32 kernel
std::vector<double> fp32c_rows(const swm_gpu_ctx *c) {
  const HostGrid &g = c->hg;
  int ny = c->ny;
  double A = c->cfg.A, dL = g.dLambda, dT = g.dTheta;
  std::vector<double> rows((size_t)ny * Q_NR);
  for (int j = 0; j < ny; j++) {
    double *r = &rows[(size_t)j * Q_NR];
    int jm = j == 0 ? ny - 1 : j - 1;
    double cE = g.cosl[GE][j], cV = g.cosl[GV][j], cU = g.cosl[GU][j], cH = g.cosl[GH][j];
    r[Q_CV] = cV;
    r[Q_DCV] = cV - g.cosl[GV][jm];
    r[Q_CU] = cU;
    r[Q_DCU] = cU - g.cosl[GU][jm];
    r[Q_FH] = g.f[GH][j];
    r[Q_RE_DL] = 1. / (A * cE * dL);
    r[Q_RE_DT] = 1. / (A * cE * dT);
    r[Q_RU_DL] = 1. / (A * cU * dL);
    r[Q_RV_DL] = 1. / (A * cV * dL);
    r[Q_RH_DL] = 1. / (A * cH * dL);
    r[Q_INV_CH] = 1. / cH;
    r[Q_PC0] = -1. / (dL * A * cE);
    r[Q_HC0] = -1. / (dL * A * cH);
    r[Q_TE] = g.tanl[GE][j] / A;
    r[Q_TH] = g.tanl[GH][j] / A;
    r[Q_TU] = g.tanl[GU][j] / A;
    r[Q_TV] = g.tanl[GV][j] / A;
  }
  return rows;
}

// the per-iteration records of the step kernel (fused32.h): record J holds
// the factors iteration J reads from rows J, J-1 and J-2 (periodic in j)
std::vector<float> fp32c_records(const swm_gpu_ctx *c) {
  const int ny = c->ny;
  const std::vector<double> r = fp32c_rows(c);
  std::vector<float> rec((size_t)ny * REC_N * 4, 0.f);
  auto q = [&](int j, int k) { return (float)r[(size_t)(((j % ny) + ny) % ny) * Q_NR + k]; };
  for (int J = 0; J < ny; J++) {
    float *o = &rec[(size_t)J * REC_N * 4];
    const float a[REC_N][4] = {
        {q(J, Q_RH_DL), q(J, Q_CU), q(J, Q_DCU), q(J, Q_INV_CH)},
        {q(J, Q_FH), 0.f, 0.f, 0.f},
        {q(J - 1, Q_TE), q(J - 1, Q_PC0), q(J, Q_TH), q(J, Q_HC0)},
        {q(J - 1, Q_TU), q(J - 1, Q_RU_DL), q(J - 1, Q_TV), q(J - 1, Q_RV_DL)},
        {q(J - 2, Q_TE), q(J - 2, Q_PC0), q(J - 1, Q_TH), q(J - 1, Q_HC0)},
        {q(J - 1, Q_CV), q(J - 1, Q_DCV), q(J - 2, Q_RE_DL), q(J - 2, Q_RE_DT)},
        {q(J - 2, Q_RU_DL), q(J - 2, Q_TU), q(J - 2, Q_TV), q(J - 2, Q_RV_DL)}};
    for (int g = 0; g < REC_N; g++)
      for (int k = 0; k < 4; k++) o[4 * g + k] = a[g][k];
  }
  return rec;
}

int march_tile_cols(int mix) { return 32 * MARCH_COLS - 2 * (mix == 2 ? 2 : 1); }

// ---- tiles of the step kernel ---------------------------------------------
//
// A warp's time grows with its rows, and a row whose 4-row window holds a
// land point (every row of a strip that contains a coast) takes the masked
// body, about 1.3 times the all-ocean one.  With equal rows per warp the
// strips along a coast finish last and set the kernel's duration.  So each
// strip is cut into row groups of equal estimated cost: a body iteration
// counts 1 when the kernel's vote will pick the all-ocean body (the same
// test on the same mask words) and `slow` otherwise; a group with k rows runs
// the iterations of rows ry0 - 1 .. ry0 + k + 1 (the look-ahead rows), and
// a group takes rows while it stays within the cost of S all-ocean rows.
// per strip and row: does the kernel's vote pick the all-ocean body there
std::vector<uint8_t> march_fast_rows(int mix, int nx, int ny, const uint16_t *m16) {
  const int H = mix == 2 ? 2 : 1, TI = march_tile_cols(mix);
  const int nstrips = (nx + TI - 1) / TI;
  auto wrap = [](int g, int n) { return ((g % n) + n) % n; };
  std::vector<uint8_t> fast((size_t)nstrips * ny), ocean(ny);
  for (int s = 0; s < nstrips; s++) {
    for (int j = 0; j < ny; j++) {
      bool all = true;
      for (int col = 0; col < 32 * MARCH_COLS && all; col++) {
        const int gi = wrap(s * TI - H + col, nx);
        all = (m16[gi + (size_t)nx * j] & 0xFFFu) == 0xFFFu;
      }
      ocean[j] = all;
    }
    for (int j = 0; j < ny; j++)
      fast[(size_t)s * ny + j] = ocean[j] && ocean[wrap(j - 1, ny)] && ocean[wrap(j - 2, ny)] && ocean[wrap(j - 3, ny)];
  }
  return fast;
}

std::vector<int2> march_tiles_cut(const std::vector<uint8_t> &fast, int ny, double S, double slow) {
  const int nstrips = (int)(fast.size() / ny);
  auto wrap = [ny](int g) { return ((g % ny) + ny) % ny; };
  const double target = S + 3.0;
  std::vector<int2> tiles;
  for (int s = 0; s < nstrips; s++) {
    const uint8_t *f = &fast[(size_t)s * ny];
    auto cost = [&](int j) { return f[wrap(j)] ? 1.0 : slow; };
    for (int ry0 = 0; ry0 < ny;) {
      // iterations of k rows: ry0 - 1 .. min(ry0 + k, ny) + 1
      double c = cost(ry0 - 1) + cost(ry0) + cost(ry0 + 1) + cost(ry0 + 2);
      int k = 1;
      while (k < 255 && ry0 + k < ny) {
        const double next = c + cost(ry0 + k + 2);
        if (next > target) break;
        c = next;
        k++;
      }
      tiles.push_back(make_int2(s, (ry0 << 8) | k));
      ry0 += k;
    }
  }
  // the groups strip after strip, four to a block (a block may take the end
  // of one strip and the start of the next); idle tiles pad the last block
  while (tiles.size() % 4) tiles.push_back(make_int2(0, 0));
  return tiles;
}

std::vector<int2> march_tiles(int mix, int nx, int ny, const uint16_t *m16, double S, double slow) {
  return march_tiles_cut(march_fast_rows(mix, nx, ny, m16), ny, S, slow);
}

// estimated cost of a tile {strip, first row << 8 | rows} as march_tiles_cut counts it
double march_tile_cost(const std::vector<uint8_t> &fast, int ny, int2 t, double slow) {
  const int k = t.y & 255, ry0 = t.y >> 8;
  const uint8_t *f = &fast[(size_t)t.x * ny];
  double c = 0.;
  for (int j = ry0 - 1; j <= std::min(ry0 + k, ny) + 1; j++) c += f[((j % ny) + ny) % ny] ? 1.0 : slow;
  return k > 0 ? c : 0.;
}

}  // namespace swm

extern "C" int swm_gpu_step_strip_columns(int mixing) { return swm::march_tile_cols(mixing); }

extern "C" int swm_gpu_plan_step_tiles(int mixing, int nx, int ny, const uint16_t *mask_words, double rows,
                                       double masked_cost, int32_t *tiles, int capacity) {
  if (nx < 1 || ny < 1 || ny >= (1 << 23) || !mask_words || rows < 1. || rows > 250. || masked_cost < 1. ||
      capacity < 0 || (capacity > 0 && !tiles))
    return -1;
  const std::vector<int2> t = swm::march_tiles(mixing, nx, ny, mask_words, rows, masked_cost);
  for (size_t k = 0; k < t.size() && (int)k < capacity; k++) {
    tiles[3 * k] = t[k].x;
    tiles[3 * k + 1] = t[k].y >> 8;
    tiles[3 * k + 2] = t[k].y & 255;
  }
  return (int)t.size();
}

namespace swm {

// the common configuration the STD variant of the step kernel serves:
// nonlinear with a linearisation, no quadratic drag, no extra forcing field,
// uniform damping, wind (if any) as row profiles
static bool march_std(const P32 &p) {
  return p.nl && p.has_mode && !p.qbf && !p.has_F && p.impl_uniform && (p.wind_rows || (!p.wind_x && !p.wind_y));
}

// Is a state of `points` array points larger than L2 (89 bytes move per
// point and step)?
bool march_state_exceeds_l2(size_t points) { return exceeds_l2(89.0 * (double)points); }

bool exceeds_l2(double bytes) {
  static long long l2 = -1;
  if (l2 < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    l2 = cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev) == cudaSuccess ? v : 0;
  }
  return bytes > (double)l2;
}

// Prefetch level of the step kernel (march_strip's PF).  A state larger than
// L2 is read from DRAM every step: 2.  Otherwise the rows are in L2 when
// steps follow one another, as in a monitored run (integ): 0; a single step
// may follow other work that evicted them, and the increments it loads last
// then wait on DRAM: 1 (measured on the 1025^2 basin: 5 % faster from a cold
// L2, 1 % slower from a warm one).  SWM_GB300_MARCH_PREFETCH=0/1/2 forces it.
// SWM_GB300_MARCH_PREFETCH=3 stages the rows through the warps' row rings
// (bulk asynchronous copies) instead, in basins at least RING_MIN_NX wide.
int march_prefetch_level(size_t points, bool integ) {
  const char *e = getenv("SWM_GB300_MARCH_PREFETCH");
  if (e && e[0] >= '0' && e[0] <= (MARCH_COLS == 1 ? '3' : '2') && e[1] == 0) return e[0] - '0';
  if (march_state_exceeds_l2(points)) return 2;
  return integ ? 0 : 1;
}

static bool g_ring_launched = false;  // a ring instance has run: march_ring_check reads the counter

// the ring instances want shared memory rather than L1 for their four
// 42 KB blocks per SM
template <class K>
static void ring_carveout(K *k) {
  cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
}

int march_ring_check() {
  if (!g_ring_launched) return SWM_GPU_OK;
  unsigned v = 0;
  SWM_CK(cudaMemcpyFromSymbol(&v, g_ring_timeouts, sizeof(v)));
  if (v) {
    set_error("FP32 step kernel: " + std::to_string(v) + " warps gave up waiting for their row copies");
    return SWM_GPU_EDEVICE;
  }
  return SWM_GPU_OK;
}

template <int MIX, bool STD, int PF>
static void launch_mix_s(const P32 &p, const MarchGrid &g, cudaStream_t st, const MarchInteg *mi) {
  if (PF == 3) {
    static bool set = false;
    if (!set) {
      ring_carveout(k_march<MIX, true, STD, PF>);
      ring_carveout(k_march<MIX, false, STD, PF>);
      set = true;
    }
    g_ring_launched = true;
  }
  if (!mi) {
    k_march<MIX, false, STD, PF><<<g.blocks, 128, 0, st>>>(p, g.tiles, MarchInteg{});
    return;
  }
  // one more block for the side jobs
  if (mi->programmatic)
    launch_programmatic(k_march<MIX, true, STD, PF>, dim3(g.blocks + 1), dim3(128), st, p, g.tiles, *mi);
  else
    k_march<MIX, true, STD, PF><<<g.blocks + 1, 128, 0, st>>>(p, g.tiles, *mi);
}

template <int MIX, bool STD>
static void launch_mix_p(const P32 &p, const MarchGrid &g, cudaStream_t st, const MarchInteg *mi) {
  const int pf = march_prefetch_level((size_t)p.nx * p.ny, mi != nullptr);
#if MARCH_COLS == 2
  P32 q = p;  // the two-column kernel takes the level at run time
  q.pf = pf;
  launch_mix_s<MIX, STD, 0>(q, g, st, mi);
#else
  if (pf == 3 && p.nx >= RING_MIN_NX) launch_mix_s<MIX, STD, 3>(p, g, st, mi);
  else if (pf >= 2) launch_mix_s<MIX, STD, 2>(p, g, st, mi);
  else if (pf == 1) launch_mix_s<MIX, STD, 1>(p, g, st, mi);
  else launch_mix_s<MIX, STD, 0>(p, g, st, mi);
#endif
}

template <int MIX>
static void launch_mix(const P32 &p, const MarchGrid &g, cudaStream_t st, const MarchInteg *mi) {
  if (march_std(p)) launch_mix_p<MIX, true>(p, g, st, mi);
  else launch_mix_p<MIX, false>(p, g, st, mi);
}

static void launch_any(const P32 &p, const MarchGrid &g, cudaStream_t st, const MarchInteg *mi = nullptr) {
  if (p.mix == 2) launch_mix<2>(p, g, st, mi);
  else if (p.mix == 1) launch_mix<1>(p, g, st, mi);
  else launch_mix<0>(p, g, st, mi);
}

// SWM_GB300_MARCH_S: rows per warp (quarters allowed), 0 when unset
double march_rows_override_f() {
  const char *e = getenv("SWM_GB300_MARCH_S");
  if (!e) return 0.;
  const double s = atof(e);
  return s >= 4. && s <= 250. ? s : 0.;
}

int march_rows_override() {
  const double s = march_rows_override_f();
  return s > 0. ? (int)s : 0;
}

// SWM_GB300_MARCH_SLOW: the masked-row cost factor, 0 when unset
double march_slow_override() {
  const char *e = getenv("SWM_GB300_MARCH_SLOW");
  if (!e) return 0.;
  double v = atof(e);
  return v >= 1. && v <= 4. ? v : 0.;
}

void march_launch(swm_gpu_ctx *c, const P32 &p, const MarchGrid &g, const MarchInteg *mi) {
  launch_any(p, g, c->stream, mi);
  c->launches++;
}

static int upload_tiles(swm_gpu_ctx *c, const std::vector<int2> &t) {
  SWM_REQUIRE(c->ny < (1 << 23), "FP32 step kernel: at most 2^23 - 1 rows (tile row index)");
  if (c->march_tiles) SWM_CK(cudaFree(c->march_tiles));
  c->march_tiles = nullptr;
  c->march_blocks = 0;
  SWM_CK(cudaMalloc((void **)&c->march_tiles, t.size() * sizeof(int2)));
  SWM_CK(cudaMemcpy(c->march_tiles, t.data(), t.size() * sizeof(int2), cudaMemcpyHostToDevice));
  c->march_blocks = (int)(t.size() / 4);
  return SWM_GPU_OK;
}

// tiles of S rows per warp, without tuning
int march_default_tiles(swm_gpu_ctx *c, const P32 &p, const uint16_t *m16, int S) {
  const double slow = march_slow_override();
  c->march_S = S;
  c->march_slow = slow > 0. ? slow : 1.;
  return upload_tiles(c, march_tiles(p.mix, p.nx, p.ny, m16, S, c->march_slow));
}

// Mean time of `reps` launches per candidate; the step reads level n0 and
// slots 1-2 and writes level n0p1 and slot 3 only, so repeating it leaves
// the model state as one launch leaves it.
int march_pick_rows(cudaStream_t st, int reps, const std::vector<int> &cands, const std::function<void(int)> &launch,
                    int *best) {
  cudaEvent_t a, b;
  SWM_CK(cudaEventCreate(&a));
  SWM_CK(cudaEventCreate(&b));
  float tbest = 1e30f;
  *best = cands.empty() ? 16 : cands[0];
  for (size_t i = 0; i < cands.size(); i++) {
    const int r = cands[i];
    launch(r);  // warm-up
    SWM_CK(cudaEventRecord(a, st));
    for (int k = 0; k < reps; k++) launch(r);
    SWM_CK(cudaEventRecord(b, st));
    SWM_CK(cudaEventSynchronize(b));
    float ms = 0.f;
    SWM_CK(cudaEventElapsedTime(&ms, a, b));
    if (ms < tbest) {
      tbest = ms;
      *best = r;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  SWM_CK(cudaGetLastError());
  return SWM_GPU_OK;
}

template <int MIX, bool STD, int PF>
static int resident_blocks_of() {  // blocks of k_march resident on the whole GPU at once
  static int b = 0;
  if (!b) {
    int per_sm = 0, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (PF == 3) ring_carveout(k_march<MIX, false, STD, PF>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_march<MIX, false, STD, PF>, 128, 0);
    b = sms * (per_sm > 0 ? per_sm : 1);
  }
  return b;
}

template <int MIX, bool STD>
static int resident_blocks_p(int pf) {
#if MARCH_COLS == 2
  (void)pf;  // one instance serves every level
  return resident_blocks_of<MIX, STD, 0>();
#else
  if (pf == 3) return resident_blocks_of<MIX, STD, 3>();
  return pf == 2 ? resident_blocks_of<MIX, STD, 2>()
                 : (pf == 1 ? resident_blocks_of<MIX, STD, 1>() : resident_blocks_of<MIX, STD, 0>());
#endif
}

template <int MIX>
static int resident_blocks_m(bool s, int pf) {
  return s ? resident_blocks_p<MIX, true>(pf) : resident_blocks_p<MIX, false>(pf);
}

static int resident_blocks(const P32 &p) {
  const bool s = march_std(p);
  int pf = march_prefetch_level((size_t)p.nx * p.ny, false);
  if (pf == 3 && p.nx < RING_MIN_NX) pf = 2;
  if (p.mix == 2) return resident_blocks_m<2>(s, pf);
  if (p.mix == 1) return resident_blocks_m<1>(s, pf);
  return resident_blocks_m<0>(s, pf);
}

// Tiles of the step kernel, by timing the step on this basin.  A kernel is
// fastest when all its warps are resident at once (one wave) and finish
// together, with as few rows each as that allows.  So for each masked-row
// cost in MARCH_TUNE_SLOW the candidate is the fewest rows per warp (in
// steps of 1/4) whose tiles fit one wave, and the same for two waves; plus
// equal groups of 16 rows.
constexpr double MARCH_TUNE_SLOW[] = {1.0, 1.2, 1.4, 1.6, 1.8, 2.0, 2.3, 2.6};

int march_autotune(swm_gpu_ctx *c, const P32 &p, const uint16_t *m16) {
  std::vector<std::vector<int2>> tabs;
  std::vector<std::pair<double, double>> params;
  const double s_env = march_rows_override_f();
  const double w_env = march_slow_override();
  const std::vector<uint8_t> fast = march_fast_rows(p.mix, p.nx, p.ny, m16);
  auto add = [&](double S, double w) {
    for (auto &q : params)
      if (q.first == S && q.second == w) return;
    params.push_back({S, w});
    tabs.push_back(march_tiles_cut(fast, p.ny, S, w));
  };
  if (s_env > 0.) {
    add(s_env, w_env > 0. ? w_env : 1.);
  } else {
    const int R = resident_blocks(p);
    add(16., 1.);
    for (double w : MARCH_TUNE_SLOW) {
      if (w_env > 0. && w != MARCH_TUNE_SLOW[0]) continue;
      const double wu = w_env > 0. ? w_env : w;
      for (int waves = 1; waves <= 2; waves++) {
        // the fewest rows (quarters) that fit: the block count falls as S grows
        int lo = 16, hi = 4 * 250;  // S = q / 4
        if (march_tiles_cut(fast, p.ny, hi / 4., wu).size() / 4 > (size_t)(waves * R)) continue;
        while (lo < hi) {
          const int mid = (lo + hi) / 2;
          if (march_tiles_cut(fast, p.ny, mid / 4., wu).size() / 4 > (size_t)(waves * R)) lo = mid + 1;
          else hi = mid;
        }
        add(lo / 4., wu);
      }
    }
  }
  int best = 0;
  if (tabs.size() > 1) {
    size_t maxn = 0;
    for (auto &t : tabs) maxn = std::max(maxn, t.size());
    int2 *d = nullptr;
    SWM_CK(cudaMalloc((void **)&d, maxn * sizeof(int2)));
    std::vector<int> idx(tabs.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (int)i;
    int uploaded = -1;
    const int rc = march_pick_rows(c->stream, 5, idx, [&](int i) {
      if (uploaded != i) {
        cudaMemcpyAsync(d, tabs[i].data(), tabs[i].size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream);
        uploaded = i;
      }
      launch_any(p, MarchGrid{d, (int)(tabs[i].size() / 4)}, c->stream);
    }, &best);
    cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (rc != SWM_GPU_OK) return rc;
  }
  c->march_rows = (int)params[best].first;
  c->march_S = params[best].first;
  c->march_slow = params[best].second;
  return upload_tiles(c, tabs[best]);
}

// ---- ensemble launch ------------------------------------------------------
template <int MIX, bool STD, int PF, bool INTEG>
static int ens_launch_m(const P32 *tab, const int4 *tiles, int ntiles, int *next, const EnsInteg *mi,
                        cudaStream_t st) {
  static int blocks = 0;
  if (!blocks) {
    int per_sm = 0, sms = 0, dev = 0;
    SWM_CK(cudaGetDevice(&dev));
    SWM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (PF == 3) ring_carveout(k_march_ens<MIX, STD, PF, INTEG>);
    SWM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_march_ens<MIX, STD, PF, INTEG>, 128, 0));
    blocks = sms * (per_sm > 0 ? per_sm : 1);
  }
  if (PF == 3) g_ring_launched = true;
  int need = (ntiles + 3) / 4;
  if (INTEG) {  // a monitored step: launched programmatically (k_ens_rows before it, k_ens_tile_sums after)
    SWM_CK(launch_programmatic(k_march_ens<MIX, STD, PF, INTEG>, dim3(need < blocks ? need : blocks), dim3(128), st,
                               tab, (const int4 *)tiles, ntiles, next, (const float2 *const *)mi->areas,
                               (double *)mi->partial));
    return SWM_GPU_OK;
  }
  k_march_ens<MIX, STD, PF, INTEG><<<need < blocks ? need : blocks, 128, 0, st>>>(
      tab, tiles, ntiles, next, mi ? mi->areas : nullptr, mi ? mi->partial : nullptr);
  return SWM_GPU_OK;
}

template <int MIX, bool STD, int PF>
static int ens_launch_i(const P32 *tab, const int4 *tiles, int ntiles, int *next, const EnsInteg *mi,
                        cudaStream_t st) {
  return mi ? ens_launch_m<MIX, STD, PF, true>(tab, tiles, ntiles, next, mi, st)
            : ens_launch_m<MIX, STD, PF, false>(tab, tiles, ntiles, next, mi, st);
}

template <int MIX, bool STD>
static int ens_launch_p(int pf, const P32 *tab, const int4 *tiles, int ntiles, int *next, const EnsInteg *mi,
                        cudaStream_t st) {
#if MARCH_COLS == 2
  (void)pf;  // the level is in the parameter blocks
  return ens_launch_i<MIX, STD, 0>(tab, tiles, ntiles, next, mi, st);
#else
  if (pf == 3) return ens_launch_i<MIX, STD, 3>(tab, tiles, ntiles, next, mi, st);
  if (pf == 2) return ens_launch_i<MIX, STD, 2>(tab, tiles, ntiles, next, mi, st);
  if (pf == 1) return ens_launch_i<MIX, STD, 1>(tab, tiles, ntiles, next, mi, st);
  return ens_launch_i<MIX, STD, 0>(tab, tiles, ntiles, next, mi, st);
#endif
}

template <int MIX>
static int ens_launch_mix(bool std_cfg, int pf, const P32 *tab, const int4 *tiles, int ntiles, int *next,
                          const EnsInteg *mi, cudaStream_t st) {
  return std_cfg ? ens_launch_p<MIX, true>(pf, tab, tiles, ntiles, next, mi, st)
                 : ens_launch_p<MIX, false>(pf, tab, tiles, ntiles, next, mi, st);
}

bool march_std_params(const P32 &p) { return march_std(p); }

int march_ens_launch(int mix, bool std_cfg, int pf, const P32 *tab, const int4 *tiles, int ntiles, int *next,
                     cudaStream_t st, const EnsInteg *mi) {
  if (mix == 2) return ens_launch_mix<2>(std_cfg, pf, tab, tiles, ntiles, next, mi, st);
  if (mix == 1) return ens_launch_mix<1>(std_cfg, pf, tab, tiles, ntiles, next, mi, st);
  return ens_launch_mix<0>(std_cfg, pf, tab, tiles, ntiles, next, mi, st);
}

}  // namespace swm
