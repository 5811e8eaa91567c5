// march2.cuh -- the FP32 step's strip march with two columns per lane.
//
// Included by march.cu.  The same row march as march_strip, with lane l
// holding columns 2l and 2l+1 of a 64-column strip as the halves of float2
// registers, so that the arithmetic of both columns runs in one packed
// FP32x2 instruction (__fadd2_rn / __fmul2_rn / __ffma2_rn, sm_100 and
// later).  Per point, that halves the floating-point instructions and the
// per-iteration work (factor records, loop control, the all-ocean vote,
// parameter and address arithmetic); loads and stores stay one per field and
// point.  An x-neighbour of a packed value is the lane's other half plus one
// shuffle: left (col 2l-1, 2l) = (shfl_up(.y), .x), right (2l+1, 2l+2) =
// (.y, shfl_down(.x)).  Mask words of the two columns travel packed in one
// 32-bit word (column 2l in bits 0-15, 2l+1 in bits 16-31), so a mask test
// gives a bit per column (0x00001 / 0x10000).
//
// Formulas and precision rules are those of march_strip (march.cu), except
// that the compensated update recovers its roundings by TwoSum rather than
// Fast2Sum (exact in more cases, three more operations); the packed
// operations are never contracted, so products that must be exact (TwoProd)
// are explicit FMAs and plain sums stay separate operations.

namespace v2 {
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 operator-(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 operator*(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 operator*(float a, float2 b) { return __fmul2_rn(make_float2(a, a), b); }
__device__ __forceinline__ float2 operator*(float2 a, float b) { return __fmul2_rn(a, make_float2(b, b)); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fma2(float a, float2 b, float2 c) { return __ffma2_rn(make_float2(a, a), b, c); }
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 div2(float2 a, float2 b) {
  return make_float2(__fdividef(a.x, b.x), __fdividef(a.y, b.y));
}
__device__ __forceinline__ float2 max2(float2 a, float b) { return make_float2(fmaxf(a.x, b), fmaxf(a.y, b)); }
// column-wise select by packed mask bits (bit 0: column 2l, bit 16: 2l+1)
__device__ __forceinline__ float2 selb(unsigned b, float2 v) {
  return make_float2((b & 1u) ? v.x : 0.f, (b >> 16) ? v.y : 0.f);
}
__device__ __forceinline__ float2 selb(unsigned b, float2 v, float2 w) {
  return make_float2((b & 1u) ? v.x : w.x, (b >> 16) ? v.y : w.y);
}
// 1 / (ocean count) per column from packed counts (0-4 per half)
__device__ __forceinline__ float2 wcnt(unsigned c) { return make_float2(rcnt(c & 0xffffu), rcnt(c >> 16)); }
__device__ __forceinline__ float2 half2w(unsigned c) {
  return make_float2((c & 0xffffu) > 1 ? 0.5f : 1.f, (c >> 16) > 1 ? 0.5f : 1.f);
}
__device__ __forceinline__ float2 shl2(float2 v) { return make_float2(__shfl_up_sync(FULL, v.y, 1), v.x); }
__device__ __forceinline__ float2 shr2(float2 v) { return make_float2(v.y, __shfl_down_sync(FULL, v.x, 1)); }

// (hi + lo + inc) * (1 - dp) as a new (hi, lo) pair, both columns
__device__ __forceinline__ void comp_damp2(float2 hi, float2 lo, float2 inc, float2 dp, float2 &nh, float2 &nl) {
  const float2 s = hi + inc;
  const float2 bb = s - hi;
  float2 e = ((hi - (s - bb)) + (inc - bb)) + lo;
  const float2 c = s * dp;
  const float2 t = s - c;
  const float2 bt = t - s;
  const float2 e2 = (s - (t - bt)) + (-c - bt);
  e = fma2(-e, dp, e + e2);
  nh = t + e;
  nl = e - (nh - t);
}
}  // namespace v2

// One warp updates rows ry0 .. ry0+S-1 of strip bx (columns bx*TI ..
// bx*TI+TI-1, TI = 64 - 2*HALO) of the basin p describes; INTEG as in
// march_strip, and the prefetch level is p.pf (march_strip's PF).
template <int MIX, bool INTEG = false, bool STD = false, int PF = 0>
__device__ __forceinline__ void march_strip2(const P32 &p, const int bx, const int ry0, const int lane, const int S,
                                             const float2 *area = nullptr, F2 *acc = nullptr) {
  using namespace v2;
  constexpr int H = MIX == 2 ? 2 : 1;
  constexpr int TI = 64 - 2 * H;
  const int nx = p.nx, ny = p.ny;
  const int c0 = 2 * lane;  // column of the strip held in .x (.y: c0 + 1)
  const int gx0 = bx * TI - H + c0;
  // columns wrap periodically in i (strips near either end read the other
  // end as their halo); the modulo keeps narrow basins in bounds too
  const int gi0 = ((gx0 % nx) + nx) % nx, gi1 = ((gx0 + 1) % nx + nx) % nx;
  const bool nl = STD || p.nl, has_mode = STD || p.has_mode, qbf = !STD && p.qbf, has_F = !STD && p.has_F;
  const bool impl_uniform = STD || p.impl_uniform, wind_rows = STD || p.wind_rows;
  const bool st0 = c0 >= H && c0 < 64 - H && gx0 < nx;
  const bool st1 = c0 + 1 >= H && c0 + 1 < 64 - H && gx0 + 1 < nx;
  const bool store_lane = st0 || st1;
  const unsigned stm = (st0 ? 1u : 0u) | (st1 ? 0x10000u : 0u);
  const float q1 = p.q1, G = p.G;
  const int pf = p.pf;  // a uniform run-time level here (PF is unused): fewer kernel instances

  float2 uh[4] = {}, ul[4] = {}, vh[4] = {}, vl[4] = {}, eh[4] = {}, el[4] = {}, he[4] = {};
  unsigned m[4] = {};
  float2 pll1[2] = {}, plt1[2] = {}, lu1[2] = {}, lv1[2] = {}, pll2[2] = {}, plt2[2] = {};
  float2 muh[4] = {}, mul[4] = {}, mvh[3] = {}, mvl[3] = {}, pot[3] = {}, ke[3] = {};
  int off[3] = {};

  auto ld2 = [&](const float *f, int o) { return make_float2(f[gi0 + o], f[gi1 + o]); };
  auto ldm = [&](int o) { return (unsigned)p.mask16[gi0 + o] | ((unsigned)p.mask16[gi1 + o] << 16); };

  int J = ry0 - 3;
  const int jend = min(ry0 + S, ny) + 2;
  int noff = nx * wrapm(J, ny);
  unsigned n_m = ldm(noff);
  float2 n_uh = ld2(p.uh0, noff), n_ul = ld2(p.ul0, noff), n_vh = ld2(p.vh0, noff), n_vl = ld2(p.vl0, noff);
  float2 n_eh = ld2(p.eh0, noff), n_el = ld2(p.el0, noff), n_he = ld2(p.He, noff);

  auto body = [&](auto fast_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
    constexpr unsigned BOTH = 0x10001u;
#define YB(m_, s_) (FAST ? BOTH : (((m_) >> (s_)) & BOTH))
#define YH(m_) YB(m_, 0)
#define YU(m_) YB(m_, 1)
#define YV(m_) YB(m_, 2)
#define YE(m_) YB(m_, 3)
#define YLV(m_) YB(m_, 6)
#define YLE(m_) YB(m_, 7)
#define SEL(b_, v_) (FAST ? (v_) : selb((b_), (v_)))
#define Y2(a_, b_) (FAST ? bc2(0.5f) : wcnt((a_) + (b_)))
#define Y4(a_, b_, c_, d_) (FAST ? bc2(0.25f) : wcnt((a_) + (b_) + (c_) + (d_)))
#define YHALF(a_, b_) (FAST ? bc2(0.5f) : half2w((a_) + (b_)))
    auto dval = [&](int a) {
      if (!nl) return he[a];
      const float2 d = he[a] + eh[a];
      return FAST ? d : selb(YE(m[a]), d, bc2(1.f));
    };
    const float4 *rec = p.rec + (size_t)wrapm(J, ny) * REC_N;
    const float4 fa = rec[REC_A], fb = rec[REC_B], fc = rec[REC_C], fd = rec[REC_D], fe = rec[REC_E],
                 ff = rec[REC_F];
    const float fh = reinterpret_cast<const float *>(rec + REC_G)[0];
    const int o = J - 2;
    const bool upd = o >= ry0 && o < ry0 + S && o < ny && store_lane;
    const int ko = off[2];
    float2 g1e = {}, g2e = {}, g1u = {}, g2u = {}, g1v = {}, g2v = {};
    float wxo = 0.f, wyo = 0.f;
    if (upd) {
      g1e = ld2(p.Ge1, ko); g2e = ld2(p.Ge2, ko); g1u = ld2(p.Gu1, ko); g2u = ld2(p.Gu2, ko);
      g1v = ld2(p.Gv1, ko); g2v = ld2(p.Gv2, ko);
      if (!INTEG && wind_rows) {
        if (p.wind_x) wxo = p.wx[o];
        if (p.wind_y) wyo = p.wy[o];
      }
    }

    // ---- row J: mass fluxes and PV; row J-1: kinetic energy ----------
    const float2 d0 = dval(0), d1 = dval(1), d2 = dval(2), d3 = dval(3);
    const float2 he_l = shl2(he[0]), eh_l = shl2(eh[0]);
    const float2 dl0 = shl2(d0), dl1 = shl2(d1), dl2 = shl2(d2);
    const float2 vh0_l = shl2(vh[0]), vl0_l = shl2(vl[0]);
    const float2 uh1_r = shr2(uh[1]), ul1_r = shr2(ul[1]);
    {
      const unsigned mm = m[0];
      {
        const unsigned a = YE(mm), b = YLE(mm);
        const float2 w = Y2(a, b);
        const float2 hs = (SEL(a, he[0]) + SEL(b, he_l)) * w;
        const float2 es = nl ? (SEL(a, eh[0]) + SEL(b, eh_l)) * w : bc2(0.f);
        const float2 a_h = hs * uh[0];
        const float2 a_l = fma2(hs, uh[0], -a_h) + fma2(hs, ul[0], es * uh[0]);
        muh[0] = SEL(YU(mm), a_h);
        mul[0] = SEL(YU(mm), a_l);
      }
      {
        const unsigned a = YE(mm), b = YE(m[1]);
        const float2 w = Y2(a, b);
        const float2 hs = (SEL(a, he[0]) + SEL(b, he[1])) * w;
        const float2 es = nl ? (SEL(a, eh[0]) + SEL(b, eh[1])) * w : bc2(0.f);
        const float2 b_h = hs * vh[0];
        const float2 b_l = fma2(hs, vh[0], -b_h) + fma2(hs, vl[0], es * vh[0]);
        mvh[0] = SEL(YV(mm), b_h);
        mvl[0] = SEL(YV(mm), b_l);
      }
      float2 pv = bc2(0.f);
      if (has_mode) {
        float2 zeta = bc2(0.f);
        if (nl) {
          const float2 bcf = FAST ? bc2(1.f) : selb(YH(mm), bc2(1.f), bc2(p.lbc));
          float2 dvdx = (bcf * fa.x) * ((vh[0] - vh0_l) + (vl[0] - vl0_l));
          float2 dudy = (bcf * q1) * fma2(fa.y, (uh[0] - uh[1]) + (ul[0] - ul[1]), fa.z * uh[1]);
          dvdx = SEL(YLV(mm) | YV(mm), dvdx);
          dudy = SEL(YU(mm) | YU(m[1]), dudy);
          zeta = fma2(-dudy, bc2(fa.w), dvdx);
        }
        const unsigned a = YE(mm), b = YLE(m[1]), c = YLE(mm), d = YE(m[1]);
        const float2 dh = ((SEL(a, d0) + SEL(b, dl1)) + (SEL(c, dl0) + SEL(d, d1))) * Y4(a, b, c, d);
        pv = div2(zeta + bc2(fh), max2(dh, 2.220446e-16f));
      }
      pot[0] = pv;
      float2 k1 = bc2(0.f);
      if (nl) {
        const float2 a = fma2(uh1_r, uh1_r, uh[1] * uh[1]);
        const float2 c = fma2(vh[0], vh[0], vh[1] * vh[1]);
        k1 = SEL(YE(m[1]), 0.25f * (a + c));
      }
      ke[0] = k1;
    }

    // ---- lateral stress: pll2 at row J-2, plt2 at row J-1 -------------
    if (MIX == 2) {
      {  // first pass, unit thickness, Ah = 1: pll1 at J-1, plt1 at J
        const unsigned m1 = m[1], m0 = m[0];
        {
          const unsigned ov = YV(m1), ovp = YV(m0);
          const float2 tE = fb.x * YHALF(ov, ovp);
          const float2 du = (uh1_r - uh[1]) + (ul1_r - ul[1]);
          const float2 dv = (vh[0] - vh[1]) + (vl[0] - vl[1]);
          pll1[0] = SEL(YE(m1), fma2(fb.y, du, fma2(q1, dv, tE * (SEL(ovp, vh[0]) + SEL(ov, vh[1])))));
        }
        {
          const unsigned ou = YU(m0), oum = YU(m1);
          const float2 tH = fb.z * YHALF(ou, oum);
          const float2 dv = (vh[0] - vh0_l) + (vl[0] - vl0_l);
          const float2 du = (uh[0] - uh[1]) + (ul[0] - ul[1]);
          plt1[0] = SEL(YH(m0), fma2(fb.w, dv, fma2(-q1, du, -(tH * (SEL(ou, uh[0]) + SEL(oum, uh[1]))))));
        }
      }
      {  // lu1, lv1 at row J-1
        const float2 pll1_l = shl2(pll1[0]), plt1_r = shr2(plt1[1]);
        const unsigned m1 = m[1];
        {
          const float2 t2 = (2.f * fc.x) * YHALF(YH(m1), YH(m[0]));
          lu1[0] = SEL(YU(m1), fma2(-fc.y, pll1[0] - pll1_l, fma2(q1, plt1[1] - plt1[0], t2 * (plt1[0] + plt1[1]))));
        }
        {
          const float2 t2 = (2.f * fc.z) * YHALF(YE(m1), YE(m[2]));
          lv1[0] = SEL(YV(m1), fma2(-fc.w, plt1_r - plt1[1], fma2(q1, pll1[0] - pll1[1], -(t2 * (pll1[0] + pll1[1])))));
        }
      }
      {  // second pass, thickness weighted, Ah = -bih
        const float2 lu1_r = shr2(lu1[1]), lv1_l = shl2(lv1[0]);
        const unsigned m2 = m[2], m1 = m[1];
        {
          const unsigned ov = YV(m2), ovp = YV(m1);
          const float2 tE = fd.x * YHALF(ov, ovp);
          const float2 s = fma2(fd.y, lu1_r - lu1[1], fma2(q1, lv1[0] - lv1[1], tE * (SEL(ovp, lv1[0]) + SEL(ov, lv1[1]))));
          pll2[0] = SEL(YE(m2), (-p.bih) * (d2 * s));
        }
        {
          const unsigned ou = YU(m1), oum = YU(m2);
          const float2 tH = fd.z * YHALF(ou, oum);
          const float2 s = fma2(fd.w, lv1[0] - lv1_l, fma2(-q1, lu1[0] - lu1[1], -(tH * (SEL(ou, lu1[0]) + SEL(oum, lu1[1])))));
          const unsigned a = YE(m1), b = YLE(m2), c = YLE(m1), d = YE(m2);
          const float2 dh = ((SEL(a, d1) + SEL(b, dl2)) + (SEL(c, dl1) + SEL(d, d2))) * Y4(a, b, c, d);
          plt2[0] = SEL(YH(m1), (-p.bih) * (dh * s));
        }
      }
    } else if (MIX == 1) {
      const float2 uh2_r = shr2(uh[2]), ul2_r = shr2(ul[2]);
      const float2 vh1_l = shl2(vh[1]), vl1_l = shl2(vl[1]);
      const unsigned m2 = m[2], m1 = m[1];
      {
        const unsigned ov = YV(m2), ovp = YV(m1);
        const float2 tE = fd.x * YHALF(ov, ovp);
        const float2 du = (uh2_r - uh[2]) + (ul2_r - ul[2]);
        const float2 dv = (vh[1] - vh[2]) + (vl[1] - vl[2]);
        const float2 s = fma2(fd.y, du, fma2(q1, dv, tE * (SEL(ovp, vh[1]) + SEL(ov, vh[2]))));
        pll2[0] = SEL(YE(m2), p.Ah * (d2 * s));
      }
      {
        const unsigned ou = YU(m1), oum = YU(m2);
        const float2 tH = fd.z * YHALF(ou, oum);
        const float2 dv = (vh[1] - vh1_l) + (vl[1] - vl1_l);
        const float2 du = (uh[1] - uh[2]) + (ul[1] - ul[2]);
        const float2 s = fma2(fd.w, dv, fma2(-q1, du, -(tH * (SEL(ou, uh[1]) + SEL(oum, uh[2])))));
        const unsigned a = YE(m1), b = YLE(m2), c = YLE(m1), d = YE(m2);
        const float2 dh = ((SEL(a, d1) + SEL(b, dl2)) + (SEL(c, dl1) + SEL(d, d2))) * Y4(a, b, c, d);
        plt2[0] = SEL(YH(m1), p.Ah * (dh * s));
      }
    }

    // ---- tendencies and compensated update of row o = J-2 ------------
    const float2 mvs1 = mvh[1] + mvl[1], mvs2 = mvh[2] + mvl[2];
    const float2 mus2 = muh[2] + mul[2], mus3 = muh[3] + mul[3];
    const float2 muh2_r = shr2(muh[2]), mul2_r = shr2(mul[2]), mus3_r = shr2(mus3);
    const float2 mvs2_l = shl2(mvs2), mvs1_l = shl2(mvs1);
    const float2 eh2_l = shl2(eh[2]), el2_l = shl2(el[2]), ke1_l = shl2(ke[1]);
    const float2 pot2_r = shr2(pot[2]);
    const float2 pll2_l = shl2(pll2[0]), plt2_r = shr2(plt2[1]);
    float2 vh2_l = {}, vh1_lo = {}, uh2_r = {}, uh3_r = {};
    if (qbf) {
      vh2_l = shl2(vh[2]);
      vh1_lo = shl2(vh[1]);
      uh2_r = shr2(uh[2]);
      uh3_r = shr2(uh[3]);
    }
    if (upd) {
      const unsigned mm = m[2];
      const int k0 = gi0 + ko, k1 = gi1 + ko;
      float2 aru, arv, are;
      if (INTEG) {
        aru = area[o];
        arv = area[ny + o];
        are = area[2 * ny + o];
      }
      float2 ge, gu, gv;
      {
        const float2 dmv = fma2(fe.x, (mvh[1] - mvh[2]) + (mvl[1] - mvl[2]), fe.y * mvs2);
        float2 g = fma2(-fe.z, (muh2_r - muh[2]) + (mul2_r - mul[2]), -(dmv * fe.w));
        if (has_F) g = g + make_float2(p.Fe[k0], p.Fe[k1]);
        ge = SEL(YE(mm), g);
      }
      {
        const float2 pv = 0.5f * (pot[1] + pot[2]);
        const float2 mv = 0.25f * ((mvs1 + mvs2_l) + (mvs1_l + mvs2));
        const float2 dE = fma2(G, (eh[2] - eh2_l) + (el[2] - el2_l), ke[1] - ke1_l);
        float2 g = fma2(pv, mv, -(dE * ff.x));
        const unsigned a = YE(mm), b = YLE(mm);
        const float2 du = (SEL(a, d2) + SEL(b, dl2)) * Y2(a, b);
        if (qbf) {
          const float2 vb = 0.25f * ((vh[1] + vh2_l) + (vh1_lo + vh[2]));
          const float2 gs = p.gsq_uniform ? bc2(p.gsq_s[0]) : make_float2(p.gsq[0][k0], p.gsq[0][k1]);
          const float2 sp = fma2(uh[2], uh[2], vb * vb);
          float2 f = gs * (make_float2(sqrtf(sp.x), sqrtf(sp.y)) * uh[2]);
          if (p.barotropic) f = div2(f, make_float2(p.Hu[k0], p.Hu[k1]));
          g = g - f;
        }
        float2 num = bc2(0.f);
        if (MIX) {
          const float2 t2 = (2.f * ff.y) * YHALF(YH(mm), YH(m[1]));
          num = fma2(-ff.x, pll2[0] - pll2_l, fma2(q1, plt2[1] - plt2[0], t2 * (plt2[0] + plt2[1])));
        }
        if (has_F) g = g + make_float2(p.Fx[k0], p.Fx[k1]);
        if (p.wind_x) {
          const float2 w = wind_rows ? bc2(p.ts_rho * (INTEG ? p.wx[o] : wxo))
                                     : p.ts_rho * make_float2(p.wx[k0], p.wx[k1]);
          if (nl) num = num + w;
          else g = g + w;
        }
        if (MIX || (p.wind_x && nl)) g = g + div2(num, du);
        gu = SEL(YU(mm), g);
      }
      {
        const float2 pv = 0.5f * (pot2_r + pot[2]);
        const float2 mu = 0.25f * (((muh2_r + mul2_r) + mus3) + (mus2 + mus3_r));
        const float2 dE = fma2(G, (eh[2] - eh[3]) + (el[2] - el[3]), ke[1] - ke[2]);
        float2 g = fma2(-pv, mu, -(dE * q1));
        const unsigned a = YE(mm), b = YE(m[3]);
        const float2 dv = (SEL(a, d2) + SEL(b, d3)) * Y2(a, b);
        if (qbf) {
          const float2 ub = 0.25f * ((uh2_r + uh[3]) + (uh[2] + uh3_r));
          const float2 gs = p.gsq_uniform ? bc2(p.gsq_s[1]) : make_float2(p.gsq[1][k0], p.gsq[1][k1]);
          const float2 sp = fma2(vh[2], vh[2], ub * ub);
          float2 f = gs * (make_float2(sqrtf(sp.x), sqrtf(sp.y)) * vh[2]);
          if (p.barotropic) f = div2(f, make_float2(p.Hv[k0], p.Hv[k1]));
          g = g - f;
        }
        float2 num = bc2(0.f);
        if (MIX) {
          const float2 t2 = (2.f * ff.z) * YHALF(YE(mm), YE(m[3]));
          num = fma2(-ff.w, plt2_r - plt2[1], fma2(q1, pll2[0] - pll2[1], -(t2 * (pll2[0] + pll2[1]))));
        }
        if (has_F) g = g + make_float2(p.Fy[k0], p.Fy[k1]);
        if (p.wind_y) {
          const float2 w = wind_rows ? bc2(p.ts_rho * (INTEG ? p.wy[o] : wyo))
                                     : p.ts_rho * make_float2(p.wy[k0], p.wy[k1]);
          if (nl) num = num + w;
          else g = g + w;
        }
        if (MIX || (p.wind_y && nl)) g = g + div2(num, dv);
        gv = SEL(YV(mm), g);
      }
      if (st0) { p.Ge3[k0] = ge.x; p.Gu3[k0] = gu.x; p.Gv3[k0] = gv.x; }
      if (st1) { p.Ge3[k1] = ge.y; p.Gu3[k1] = gu.y; p.Gv3[k1] = gv.y; }
      float2 dpu, dpv, dpe;
      if (impl_uniform) {
        dpu = bc2(p.dp_s[0]); dpv = bc2(p.dp_s[1]); dpe = bc2(p.dp_s[2]);
      } else {
        dpu = make_float2(p.dp[0][k0], p.dp[0][k1]);
        dpv = make_float2(p.dp[1][k0], p.dp[1][k1]);
        dpe = make_float2(p.dp[2][k0], p.dp[2][k1]);
      }
      const float2 ince = p.dt * fma2(p.ab0, g1e, fma2(p.ab1, g2e, p.ab2 * ge));
      const float2 incu = p.dt * fma2(p.ab0, g1u, fma2(p.ab1, g2u, p.ab2 * gu));
      const float2 incv = p.dt * fma2(p.ab0, g1v, fma2(p.ab1, g2v, p.ab2 * gv));
      float2 nh, nlo;
      comp_damp2(eh[2], el[2], ince, dpe, nh, nlo);
      if (nl) {
        const float2 lim = bc2(p.minD) - he[2];
        if (nh.x < lim.x) { nh.x = lim.x; nlo.x = 0.f; }
        if (nh.y < lim.y) { nh.y = lim.y; nlo.y = 0.f; }
      }
      if (st0) { p.eh1[k0] = nh.x; p.el1[k0] = nlo.x; }
      if (st1) { p.eh1[k1] = nh.y; p.el1[k1] = nlo.y; }
      if (INTEG) {
        const unsigned w = YE(mm) & stm;
        F2 x, sq;
        if (w & 1u) {
          x.h = nh.x; x.l = nlo.x;
          acc[0].add_prod(are, x);
          sq_pair(nh.x, nlo.x, sq.h, sq.l);
          acc[1].add_prod(are, sq);
        }
        if (w >> 16) {
          x.h = nh.y; x.l = nlo.y;
          acc[0].add_prod(are, x);
          sq_pair(nh.y, nlo.y, sq.h, sq.l);
          acc[1].add_prod(are, sq);
        }
      }
      comp_damp2(uh[2], ul[2], incu, dpu, nh, nlo);
      if (st0) { p.uh1[k0] = nh.x; p.ul1[k0] = nlo.x; }
      if (st1) { p.uh1[k1] = nh.y; p.ul1[k1] = nlo.y; }
      if (INTEG) {
        const unsigned w = YU(mm) & stm;
        F2 sq;
        if (w & 1u) { sq_pair(nh.x, nlo.x, sq.h, sq.l); acc[2].add_prod(aru, sq); }
        if (w >> 16) { sq_pair(nh.y, nlo.y, sq.h, sq.l); acc[2].add_prod(aru, sq); }
      }
      comp_damp2(vh[2], vl[2], incv, dpv, nh, nlo);
      if (st0) { p.vh1[k0] = nh.x; p.vl1[k0] = nlo.x; }
      if (st1) { p.vh1[k1] = nh.y; p.vl1[k1] = nlo.y; }
      if (INTEG) {
        const unsigned w = YV(mm) & stm;
        F2 sq;
        if (w & 1u) { sq_pair(nh.x, nlo.x, sq.h, sq.l); acc[3].add_prod(arv, sq); }
        if (w >> 16) { sq_pair(nh.y, nlo.y, sq.h, sq.l); acc[3].add_prod(arv, sq); }
      }
    }
#undef YB
#undef YH
#undef YU
#undef YV
#undef YE
#undef YLV
#undef YLE
#undef SEL
#undef Y2
#undef Y4
#undef YHALF
  };

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
    m[0] = n_m; uh[0] = n_uh; ul[0] = n_ul; vh[0] = n_vh; vl[0] = n_vl;
    eh[0] = n_eh; el[0] = n_el; he[0] = n_he;
    off[0] = noff;
    if (J + 1 < jend) {  // prefetch row J+1
      noff = nx * wrapm(J + 1, ny);
      n_m = ldm(noff);
      n_uh = ld2(p.uh0, noff); n_ul = ld2(p.ul0, noff); n_vh = ld2(p.vh0, noff); n_vl = ld2(p.vl0, noff);
      n_eh = ld2(p.eh0, noff); n_el = ld2(p.el0, noff); n_he = ld2(p.He, noff);
    }
    if (pf >= 1) {
      // one prefetch per lane covers both of its columns (adjacent words)
      if (pf == 2 && J + 2 < jend) {
        const int k2 = gi0 + nx * wrapm(J + 2, ny);
        prefetch_l2(p.mask16 + k2);
        prefetch_l2(p.uh0 + k2); prefetch_l2(p.ul0 + k2); prefetch_l2(p.vh0 + k2); prefetch_l2(p.vl0 + k2);
        prefetch_l2(p.eh0 + k2); prefetch_l2(p.el0 + k2); prefetch_l2(p.He + k2);
      }
      if (store_lane && J - 1 >= ry0 && J - 1 < ry0 + S && J - 1 < ny) {
        const int k1 = gi0 + off[1];
        prefetch_l2(p.Ge1 + k1); prefetch_l2(p.Ge2 + k1); prefetch_l2(p.Gu1 + k1);
        prefetch_l2(p.Gu2 + k1); prefetch_l2(p.Gv1 + k1); prefetch_l2(p.Gv2 + k1);
      }
    }
    if (J < ry0 - 1) continue;
    const bool interior = __all_sync(FULL, (m[0] & m[1] & m[2] & m[3] & 0x0FFF0FFFu) == 0x0FFF0FFFu);
    if (interior) body(std::true_type{});
    else body(std::false_type{});
  }
}
