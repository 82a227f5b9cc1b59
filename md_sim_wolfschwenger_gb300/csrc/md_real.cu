// md_real.cu -- kernel (b): real-space Ewald sum of the dipolar field, force
// and pressure, the hard-core overlap push and the short-range coating
// potentials.  Restates, per particle instead of per listed pair:
//   CompInteractVecs overlap handling   src/interaction.cpp:104-129
//   CompDipInteractEwaldR + EvalPressTensLR  src/interaction.cpp:383-422,
//                                         src/postprocessing.cpp:195-200
//   CompDipFieldEwaldR                  src/interaction.cpp:555-582
//   CompSterRep/CompElectrostatRep/CompForceVdW + EvalPressTensSR
//                                       src/interaction.cpp:766-832,
//                                       src/simulation.cpp:648-676
//
// Neighbour search.  The reference lists every pair with r < rc each step
// (all N(N-1)/2 pairs, CompInteractVecs).  Here a Verlet list with a skin
// holds, for each cell-sorted particle, the particles within rc + skin at the
// last build; it is rebuilt (on the device, inside the step) when some
// particle has moved more than skin/2 since then, so every pair that is now
// within rc is in the list.  Each evaluation tests the exact distance
// against rc like the reference.  Build: one warp per particle walks the rows
// of its cell stencil; lane r computes row r's cell range, culled to the
// cells that intersect the search sphere; lanes test 32 candidates at a time
// (next 32 prefetched) and a ballot compacts the hits (count pass, prefix
// sum, fill pass).  If the list does not fit its capacity the evaluation
// falls back to that scan directly, with in-range pairs compacted into a
// per-warp shared-memory queue (correct, slower); the host then grows the
// list.
//
// Evaluation: one warp per particle; lanes take list entries 32 at a time,
// gather the neighbour's coordinates and moment, and run the pair maths
// (erfc, exp, ~90 flops).  Per-lane sums are reduced with warp shuffles.
//
// Geometry (mixed path): 32-bit fixed-point coordinates (2^32 per box
// length); their wrapping difference is the exact minimum image, converted
// to FP32 once (relative error ~6e-8 in r at any distance).  The FP64 path
// uses FP64 box coordinates and the reference's fold (d > L/2 -> d - L,
// d < -L/2 -> d + L), with an FP32 pre-test that has a small margin.
//
// erfc on the mixed path: the Chebyshev fit erfcc of Numerical Recipes
// (Press et al., 2nd ed., section 6.2), relative error < 1.2e-7 for x >= 0,
// written as t exp(-x^2) exp(P(t)) so that exp(-x^2) is shared with the
// Gaussian term; exponentials with __expf.  The FP64 path calls erfc/exp.
//
// Overlap push: CompInteractVecs moves cores apart in place while it walks
// the pairs, so later pairs see moved positions.  Here every overlap is
// resolved from the same starting positions (Jacobi): particle i collects
// -1/2 (dCont - r) r_hat_ij over its overlapping neighbours, r is clamped to
// dCont for the Ewald terms, and the displacement is applied with the
// translation step.  For configurations without overlaps the two agree.
//
// Roofline: FP32/SFU issue bound.  Algorithmic FLOPs per unordered in-range
// pair (counted from the reference formula): 113 full, 58 field only.
#include <algorithm>

#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kRealWarps = 8;  // warps (particles) per block: list build, full pass, packed launches
// warps per block of the single-system field pass (its packed pair maths
// needs fewer registers; smaller blocks give finer occupancy steps)
constexpr int kFieldWarps = 4;

template <typename T>
struct Acc {
  T b0 = 0, b1 = 0, b2 = 0, f0 = 0, f1 = 0, f2 = 0, o0 = 0, o1 = 0, o2 = 0, p0 = 0, p1 = 0, p2 = 0;
  int np = 0;  // in-range pairs seen by this lane
};

// Numerical Recipes erfcc: erfc(z) = t exp(-z^2 + P(t)), t = 1/(1 + z/2).
__device__ __forceinline__ float erfc_nr(float z, float ez2) {
  const float t = __fdividef(1.0f, fmaf(0.5f, z, 1.0f));
  float q = 0.17087277f;
  q = fmaf(q, t, -0.82215223f);
  q = fmaf(q, t, 1.48851587f);
  q = fmaf(q, t, -1.13520398f);
  q = fmaf(q, t, 0.27886807f);
  q = fmaf(q, t, -0.18628806f);
  q = fmaf(q, t, 0.09678418f);
  q = fmaf(q, t, 0.37409196f);
  q = fmaf(q, t, 1.00002368f);
  q = fmaf(q, t, -1.26551223f);
  return t * ez2 * __expf(q);
}

// Ewald pair terms for the pair vector (dx, dy, dz) from i to j (r2 < rc2).
template <typename T, bool FULL, bool COAT>
__device__ __forceinline__ void pair_terms(const RealParams& p, T dx, T dy, T dz, T r2, const typename V4<T>::t& mi,
                                           const typename V4<T>::t& mj, int oi, int oj, Acc<T>& a) {
  a.np++;
  T ir0, r0;
  if constexpr (std::is_same<T, float>::value) {
    ir0 = rsqrtf(r2);
    r0 = r2 * ir0;
  } else {
    ir0 = rsqrt(r2);
    r0 = r2 * ir0;
  }
  const T ux = dx * ir0, uy = dy * ir0, uz = dz * ir0;
  T r = r0, ire = ir0;
  const T dcont = mi.w + mj.w + (T)p.cont_eps;
  if (r < dcont) {
    if constexpr (FULL) {
      const T h = (T)0.5 * (dcont - r);
      a.o0 -= h * ux;
      a.o1 -= h * uy;
      a.o2 -= h * uz;
    }
    r = dcont;
    if constexpr (std::is_same<T, float>::value)
      ire = __fdividef(1.0f, r);
    else
      ire = 1.0 / r;
  }
  const T ire2 = ire * ire;
  const T re2 = r * r;
  T e, erfcv;
  if constexpr (std::is_same<T, float>::value) {
    e = __expf(-(float)p.al2 * re2);
    erfcv = erfc_nr((float)p.alpha * r, e);
  } else {
    e = exp(-p.al2 * re2);
    erfcv = erfc(p.alpha * r);
  }
  const T t = (T)p.c2a * e * ire2;
  const T a1 = erfcv * ire2 * ire + t;
  const T a2 = (T)3 * a1 * ire2 + (T)2 * (T)p.al2 * t;
  const T d1 = mi.x * ux + mi.y * uy + mi.z * uz;
  const T d2 = mj.x * ux + mj.y * uy + mj.z * uz;
  const T c1 = a2 * d2 * re2;
  a.b0 += c1 * ux - a1 * mj.x;
  a.b1 += c1 * uy - a1 * mj.y;
  a.b2 += c1 * uz - a1 * mj.z;
  if constexpr (FULL) {
    const T a3 = (T)5 * a2 * ire2 + (T)4 * (T)p.al4 * t;
    const T m12 = mi.x * mj.x + mi.y * mj.y + mi.z * mj.z;
    const T s1 = (a2 * m12 - a3 * d1 * d2 * re2) * r;
    const T s2 = a2 * r;
    const T vx = s1 * ux + s2 * (d2 * mi.x + d1 * mj.x);
    const T vy = s1 * uy + s2 * (d2 * mi.y + d1 * mj.y);
    const T vz = s1 * uz + s2 * (d2 * mi.z + d1 * mj.z);
    a.f0 -= vx;
    a.f1 -= vy;
    a.f2 -= vz;
    a.p0 += r * ux * vy;
    a.p1 += r * ux * vz;
    a.p2 += r * uy * vz;
    if constexpr (COAT) {
      // Coating potentials for pairs inside rCutSR (intRangeSR uses the
      // unclamped distance, interaction.cpp:115), evaluated in FP64 with the
      // clamped distance like the reference's list length.
      if ((double)r2 < p.rcut_sr2) {
        double rd = sqrt((double)dx * dx + (double)dy * dy + (double)dz * dz);
        const double ri = p.rMag_u[oi], rj = p.rMag_u[oj];
        const double dc = ri + rj + p.cont_eps;
        if (rd < dc) rd = dc;
        // steric repulsion is asymmetric: dDelta and the prefactor use the
        // pair's lower particle index as "idx1" (interaction.cpp:768-775)
        const double ra = oi < oj ? ri : rj, rb = oi < oj ? rj : ri;
        const double dDelta = 2.0 * (ra + p.eff_len);
        double s = rd <= dDelta ? (2.0 * rb / (ra + rb)) * p.ster * ra * ra * log(dDelta / rd) : 0.0;
        s += (ri * rj / (ri + rj)) * p.elec * exp(-p.kappa * (rd - ri - rj));
        const double g1 = (rd - ri - rj) * (rd + ri + rj), g2 = rd * rd - (ri - rj) * (ri - rj);
        const double c4 = 4.0 * ri * rj;
        s += -p.vdw * rd * (c4 * c4 * c4) / (6.0 * g1 * g1 * g2 * g2);
        const T sv = (T)s;
        a.f0 -= sv * ux;
        a.f1 -= sv * uy;
        a.f2 -= sv * uz;
        a.p0 += r * ux * sv * uy;
        a.p1 += r * ux * sv * uz;
        a.p2 += r * uy * sv * uz;
      }
    }
  }
}

// ------------------------------------------------- packed pair terms (FP32)
// Two pairs at once in the halves of float2 operations (Blackwell's packed
// FP32 instructions: one issue slot for two FMAs, the FMA rate unchanged), for
// the mixed path's list loop, which gathers two neighbours per lane and
// iteration.  The per-pair arithmetic is the one of pair_terms (same
// operations and rounding per half); special functions stay scalar.
__device__ __forceinline__ float2 pk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 pk1(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

struct Acc2 {
  float2 b0 = {0.f, 0.f}, b1 = {0.f, 0.f}, b2 = {0.f, 0.f}, f0 = {0.f, 0.f}, f1 = {0.f, 0.f}, f2 = {0.f, 0.f};
  float2 p0 = {0.f, 0.f}, p1 = {0.f, 0.f}, p2 = {0.f, 0.f};
};

// Single-instruction approximations (PTX ex2/rsqrt/rcp .approx.ftz); their
// arguments here are never subnormal, so flushing changes nothing.
__device__ __forceinline__ float ex2_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// erfc polynomial of Numerical Recipes' erfcc (the one of erfc_nr) times
// log2(e), so that 2^q replaces exp(q); the coefficients stay below 2 in
// magnitude, so the scaling costs no precision.
__host__ __device__ constexpr float erfc_c(double c) { return (float)(c * 1.4426950408889634); }

// Pairs A and B: fixed-point pair vectors (dxf..), r2f = |d_fix|^2, the
// neighbour moments ma, mb; inA, inB: the pair is within rc.  Pairs outside
// get a harmless distance and weight 0.  wA, wB: the pair's Ewald field,
// force and pressure go into the sums (in range and not a strong pair, whose
// terms the FP64 kernels add; the overlap push follows inA, inB).  Same
// formulas as pair_terms, with the field sums of the field-only pass as two
// FMAs per component.
template <bool FULL>
__device__ __forceinline__ void pair_terms2(const PairK& K, float wdc, float2 dxf, float2 dyf, float2 dzf, float2 r2f,
                                            bool inA, bool inB, bool wA, bool wB, float rc2_fix, const float4& mi,
                                            const float4& ma, const float4& mb, Acc<float>& a, Acc2& a2) {
  const float sc = 2.3283064365386963e-10f;  // 2^-32 (exact scaling)
  r2f = pk(inA ? r2f.x : rc2_fix, inB ? r2f.y : rc2_fix);
  a.np += (int)inA + (int)inB;
  float2 irf = pk(rsqrt_ftz(r2f.x), rsqrt_ftz(r2f.y));  // 1 / r_fix
  float2 rfx = mul2(r2f, irf);  // r_fix
  float2 r = mul2(rfx, pk1(sc));
  const float2 dcont = pk(wdc + ma.w, wdc + mb.w);
  const bool ovA = inA && r.x < dcont.x, ovB = inB && r.y < dcont.y;
  if (ovA || ovB) {  // rare: clamp overlapping pairs to contact
    const float s32 = 4294967296.0f;
    // push along the unit vector d / r; then the pair vector itself is
    // rescaled to the contact length, which the assembly below uses
    if (ovA) {
      if constexpr (FULL) {
        const float h = 0.5f * (dcont.x - r.x) * irf.x;
        a.o0 -= h * dxf.x;
        a.o1 -= h * dyf.x;
        a.o2 -= h * dzf.x;
      }
      const float g = dcont.x * s32 * irf.x;
      dxf.x *= g;
      dyf.x *= g;
      dzf.x *= g;
      r.x = dcont.x;
      rfx.x = dcont.x * s32;
      irf.x = rcp_ftz(rfx.x);
      r2f.x = rfx.x * rfx.x;
    }
    if (ovB) {
      if constexpr (FULL) {
        const float h = 0.5f * (dcont.y - r.y) * irf.y;
        a.o0 -= h * dxf.y;
        a.o1 -= h * dyf.y;
        a.o2 -= h * dzf.y;
      }
      const float g = dcont.y * s32 * irf.y;
      dxf.y *= g;
      dyf.y *= g;
      dzf.y *= g;
      r.y = dcont.y;
      rfx.y = dcont.y * s32;
      irf.y = rcp_ftz(rfx.y);
      r2f.y = rfx.y * rfx.y;
    }
  }
  const float2 ire = mul2(irf, pk1(4294967296.0f));  // 1 / r
  const float2 ire2 = mul2(ire, ire);
  const float2 ee = mul2(pk1(K.ke), r2f);
  const float2 e = pk(ex2_ftz(ee.x), ex2_ftz(ee.y));  // exp(-alpha^2 r^2)
  const float2 den = fma2(pk1(K.kz), rfx, pk1(1.0f));
  const float2 tt = pk(rcp_ftz(den.x), rcp_ftz(den.y));
  float2 q = pk1(erfc_c(0.17087277));
  q = fma2(q, tt, pk1(erfc_c(-0.82215223)));
  q = fma2(q, tt, pk1(erfc_c(1.48851587)));
  q = fma2(q, tt, pk1(erfc_c(-1.13520398)));
  q = fma2(q, tt, pk1(erfc_c(0.27886807)));
  q = fma2(q, tt, pk1(erfc_c(-0.18628806)));
  q = fma2(q, tt, pk1(erfc_c(0.09678418)));
  q = fma2(q, tt, pk1(erfc_c(0.37409196)));
  q = fma2(q, tt, pk1(erfc_c(1.00002368)));
  q = fma2(q, tt, pk1(erfc_c(-1.26551223)));
  const float2 erfcv = mul2(mul2(tt, e), pk(ex2_ftz(q.x), ex2_ftz(q.y)));
  const float2 t = mul2(mul2(pk1(K.c2a), e), ire2);
  if constexpr (FULL) {
    // field + force: packed coefficients, then each pair assembled in scalar
    // code (as pair_terms), which keeps fewer values live.  The assembly uses
    // the pair vector d = r u itself: B = a2 (mj.d) d - a1 mj, F_ij = (a2 m12
    // - a3 (mi.d)(mj.d)) d + a2 ((mj.d) mi + (mi.d) mj), P += d_x F_y, ...
    // (no normalisation, fewer products of r)
    const float2 w = pk(wA ? 1.f : 0.f, wB ? 1.f : 0.f);
    const float2 a1 = mul2(fma2(mul2(erfcv, ire2), ire, t), w);
    const float2 tw = mul2(t, w);
    const float2 a2c = fma2(mul2(pk1(3.f), a1), ire2, mul2(pk1(K.al2x2), tw));
    const float2 a3 = fma2(mul2(pk1(5.f), a2c), ire2, mul2(pk1(K.al4x4), tw));
    const float2 dvx = mul2(dxf, pk1(sc)), dvy = mul2(dyf, pk1(sc)), dvz = mul2(dzf, pk1(sc));  // box units
    auto assemble = [&](float a1s, float a2s, float a3s, float dx, float dy, float dz, const float4& mj) {
      // dot products in scalar code: packed, they would first pair up the
      // two neighbours' moment components
      const float D1 = fmaf(mi.z, dz, fmaf(mi.y, dy, mi.x * dx));
      const float D2 = fmaf(mj.z, dz, fmaf(mj.y, dy, mj.x * dx));
      const float e2 = a2s * D2;
      a.b0 = fmaf(e2, dx, fmaf(-a1s, mj.x, a.b0));
      a.b1 = fmaf(e2, dy, fmaf(-a1s, mj.y, a.b1));
      a.b2 = fmaf(e2, dz, fmaf(-a1s, mj.z, a.b2));
      const float m12 = fmaf(mi.z, mj.z, fmaf(mi.y, mj.y, mi.x * mj.x));
      const float t1 = fmaf(-a3s * D1, D2, a2s * m12);
      const float e1 = a2s * D1;
      const float vx = fmaf(t1, dx, fmaf(e2, mi.x, e1 * mj.x));
      const float vy = fmaf(t1, dy, fmaf(e2, mi.y, e1 * mj.y));
      const float vz = fmaf(t1, dz, fmaf(e2, mi.z, e1 * mj.z));
      a.f0 -= vx;
      a.f1 -= vy;
      a.f2 -= vz;
      a.p0 = fmaf(dx, vy, a.p0);
      a.p1 = fmaf(dx, vz, a.p1);
      a.p2 = fmaf(dy, vz, a.p2);
    };
    assemble(a1.x, a2c.x, a3.x, dvx.x, dvy.x, dvz.x, ma);
    assemble(a1.y, a2c.y, a3.y, dvx.y, dvy.y, dvz.y, mb);
  } else {
    // B += a2 (mj.d) d - a1 mj with d the pair vector in fixed-point units
    // (a2 (mj.u) r^2 u), the weight negated (wn = -w): a1n = -a1, and the
    // 2^-64 of the fixed-point units folded into a2s
    const float2 mjx = pk(ma.x, mb.x), mjy = pk(ma.y, mb.y), mjz = pk(ma.z, mb.z);
    const float2 d2 = fma2(mjz, dzf, fma2(mjy, dyf, mul2(mjx, dxf)));
    const float2 wn = pk(wA ? -1.f : 0.f, wB ? -1.f : 0.f);
    const float2 a1n = mul2(fma2(mul2(erfcv, ire2), ire, t), wn);
    const float2 a2s = fma2(mul2(pk1(K.ka2n), a1n), ire2, mul2(pk1(K.kt2n), mul2(t, wn)));
    const float2 c1 = mul2(a2s, d2);
    a2.b0 = fma2(c1, dxf, fma2(a1n, mjx, a2.b0));
    a2.b1 = fma2(c1, dyf, fma2(a1n, mjy, a2.b1));
    a2.b2 = fma2(c1, dzf, fma2(a1n, mjz, a2.b2));
  }
}

// Own coordinates of sorted particle k.
template <typename T>
struct Self {
  int4 si;
  double4_32a di;
  float x, y, z;
  int oi;
};

template <typename T, bool COAT>
__device__ __forceinline__ Self<T> load_self(const RealParams& p, int k) {
  Self<T> s;
  s.si = make_int4(0, 0, 0, 0);
  s.di = make_double4_32a(0, 0, 0, 0);
  if constexpr (std::is_same<T, float>::value) {
    s.si = p.s.xi[k];
    const float sc = 2.3283064365386963e-10f;
    s.x = (float)s.si.x * sc;
    s.y = (float)s.si.y * sc;
    s.z = (float)s.si.z * sc;
    s.oi = s.si.w;
  } else {
    s.di = p.s.xd[k];
    const float4 f = p.s.xf[k];
    s.x = f.x;
    s.y = f.y;
    s.z = f.z;
    s.oi = COAT ? p.s.perm[k] : 0;
  }
  return s;
}

// Walks the cell-stencil rows of particle k and calls visit(in, j, dx, dy, dz)
// for every batch of 32 candidates (warp-synchronous; `in` marks candidates
// within the search radius; dx.. is the pair vector on the mixed path).
template <typename T, typename V>
__device__ __forceinline__ void scan_rows(const RealParams& p, int k, int lane, const Self<T>& me, double r2box,
                                          V&& visit) {
  constexpr bool F32 = std::is_same<T, float>::value;
  const int ncx = p.grid.ncx, m = p.grid.reach, side = 2 * m + 1, R = side * side;
  const int cell = p.s.cell[k];
  const int cx = cell % ncx, cy = (cell / ncx) % ncx, cz = cell / (ncx * ncx);
  const float inv = 1.0f / (float)ncx;
  const double rr = sqrt(r2box);
  const float rt = (float)(rr * (1.0 + 1e-6) + 2e-7);
  const float rct2 = rt * rt;                                          // culling / FP64 pre-test
  const float r2fix = (float)(r2box * 18446744073709551616.0);         // (r / (L 2^-32))^2
  const int* cs = p.s.cell_start;
  auto scan = [&](int s, int e) {
    if (s >= e) return;
    if constexpr (F32) {
      const float sc = 2.3283064365386963e-10f;
      int4 nxt = s + lane < e ? p.s.xi[s + lane] : make_int4(0, 0, 0, 0);
      for (int j0 = s; j0 < e; j0 += 32) {
        const int j = j0 + lane;
        const int4 sj = nxt;
        if (j0 + 32 + lane < e) nxt = p.s.xi[j0 + 32 + lane];
        const float dx = (float)(sj.x - me.si.x), dy = (float)(sj.y - me.si.y), dz = (float)(sj.z - me.si.z);
        const bool in = j < e && j != k && dx * dx + dy * dy + dz * dz < r2fix;
        visit(in, j, dx * sc, dy * sc, dz * sc);
      }
    } else {
      float4 nxt = s + lane < e ? p.s.xf[s + lane] : make_float4(0, 0, 0, 0);
      for (int j0 = s; j0 < e; j0 += 32) {
        const int j = j0 + lane;
        const float4 xj = nxt;
        if (j0 + 32 + lane < e) nxt = p.s.xf[j0 + 32 + lane];
        float dx = xj.x - me.x, dy = xj.y - me.y, dz = xj.z - me.z;
        dx -= rintf(dx);
        dy -= rintf(dy);
        dz -= rintf(dz);
        const bool in = j < e && j != k && dx * dx + dy * dy + dz * dz < rct2;
        visit(in, j, 0.f, 0.f, 0.f);
      }
    }
  };
  for (int rb = 0; rb < R; rb += 32) {
    const int r = rb + lane;
    int a0 = 0, b0 = 0, a1 = 0, b1 = 0;
    if (r < R) {
      const int dy = r % side - m, dz = r / side - m;
      const int uy = cy + dy, uz = cz + dz;
      int xlo = cx - m, xhi = cx + m;
      bool ok = true;
      if (ncx > 1) {
        const float ylo = uy * inv - 0.5f, yhi = ylo + inv, zlo = uz * inv - 0.5f, zhi = zlo + inv;
        const float ey = fmaxf(0.f, fmaxf(ylo - me.y, me.y - yhi));
        const float ez = fmaxf(0.f, fmaxf(zlo - me.z, me.z - zhi));
        const float d2 = ey * ey + ez * ez;
        ok = d2 < rct2;
        if (ok) {
          const float w = sqrtf(rct2 - d2);
          xlo = max(xlo, (int)floorf((me.x - w + 0.5f) * ncx));
          xhi = min(xhi, (int)floorf((me.x + w + 0.5f) * ncx));
        }
      }
      if (ok && xlo <= xhi) {
        const int wy = (uy + ncx) % ncx, wz = (uz + ncx) % ncx;
        const int base = (wz * ncx + wy) * ncx;
        if (xlo < 0) {
          a0 = cs[base + xlo + ncx];
          b0 = cs[base + ncx];
          a1 = cs[base];
          b1 = cs[base + xhi + 1];
        } else if (xhi >= ncx) {
          a0 = cs[base + xlo];
          b0 = cs[base + ncx];
          a1 = cs[base];
          b1 = cs[base + xhi - ncx + 1];
        } else {
          a0 = cs[base + xlo];
          b0 = cs[base + xhi + 1];
        }
      }
    }
    const int nr = min(32, R - rb);
    for (int q = 0; q < nr; q++) {
      const int s0 = __shfl_sync(kFull, a0, q), e0 = __shfl_sync(kFull, b0, q);
      const int s1 = __shfl_sync(kFull, a1, q), e1 = __shfl_sync(kFull, b1, q);
      scan(s0, e0);
      scan(s1, e1);
    }
  }
}

// ------------------------------------------------------- neighbour list

// Count (FILL = false) or write (FILL = true) the neighbours within rc + skin.
// On the mixed path with strong pairs on, each neighbour is also classified
// (|mu_k|^2 |mu_j|^2 > strong_w4sq r^8 at this build): strong entries carry
// the sign bit in the Verlet list and are copied, as (k, j), into the
// strong list (unless that list overflowed in the count).
template <typename T, bool FILL>
__device__ __forceinline__ void nbr_build(const RealParams& p, int bx) {
  if (!p.flags->rebuild) return;
  if (FILL && p.flags->overflow) return;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = bx * kRealWarps + wib;
  if (k >= p.n) return;
  const Self<T> me = load_self<T, false>(p, k);
  constexpr bool F32 = std::is_same<T, float>::value;
  const bool cls = F32 && p.strong;
  const float4* gmu = (const float4*)p.s.mu;
  float mi2 = 0.f;
  if (cls) {
    const float4 m = gmu[k];
    mi2 = m.x * m.x + m.y * m.y + m.z * m.z;
  }
  const bool sfill = FILL && cls && !p.flags->soverflow;
  int cnt = 0, scnt = 0;
  int* out = FILL ? p.nbr + p.nbr_off[k] : nullptr;
  int2* sout = sfill ? p.snbr + p.snbr_off[k] : nullptr;
  scan_rows<T>(p, k, lane, me, p.rl2, [&](bool in, int j, float dx, float dy, float dz) {
    bool st = false;
    if (cls && in) {
      const float4 mj = gmu[j];
      const float r2 = dx * dx + dy * dy + dz * dz, r4 = r2 * r2;
      st = mi2 * (mj.x * mj.x + mj.y * mj.y + mj.z * mj.z) > p.strong_w4sq * (r4 * r4);
    }
    const unsigned mask = __ballot_sync(kFull, in);
    const unsigned smask = __ballot_sync(kFull, st);
    if (FILL && in) out[cnt + __popc(mask & lanemask_lt())] = (sfill && st) ? (int)((unsigned)j | 0x80000000u) : j;
    if (sfill && st) sout[scnt + __popc(smask & lanemask_lt())] = make_int2(k, j);
    cnt += __popc(mask);
    scnt += __popc(smask);
  });
  if (!FILL && lane == 0) {
    p.nbr_cnt[k] = cnt;
    if (cls) p.snbr_cnt[k] = scnt;
  }
}

// Exclusive scan of cnt[0, n) into off[0, n] by one block (every thread
// calls it); returns the total to every thread.  Offsets saturate at
// INT_MAX (the list is then flagged as overflowing).
__device__ __forceinline__ long long block_scan_counts(const int* cnt, int* off, int n) {
  __shared__ long long wsum[32];
  __shared__ long long total;
  const int t = threadIdx.x, nt = blockDim.x;
  const int per = (n + nt - 1) / nt;
  const int b = t * per, e = min(n, b + per);
  long long local = 0;
  for (int i = b; i < e; i++) local += cnt[i];
  const int lane = t & 31, w = t >> 5;
  long long incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long v = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const long long v = lane < (nt >> 5) ? wsum[lane] : 0;
    long long inc2 = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long u = __shfl_up_sync(kFull, inc2, o);
      if (lane >= o) inc2 += u;
    }
    wsum[lane] = inc2 - v;
  }
  __syncthreads();
  long long run = wsum[w] + incl - local;
  for (int i = b; i < e; i++) {
    off[i] = (int)min(run, (long long)0x7fffffff);
    run += cnt[i];
  }
  if (t == nt - 1) {
    off[n] = (int)min(run, (long long)0x7fffffff);
    total = run;
  }
  __syncthreads();
  const long long r = total;
  __syncthreads();  // the shared scratch is reused by a second call
  return r;
}

// Offsets of the Verlet list (and of the strong list); flags overflow.
__device__ __forceinline__ void nbr_scan(const RealParams& p) {
  StepFlags* flags = p.flags;
  if (!flags->rebuild) return;
  const long long tot = block_scan_counts(p.nbr_cnt, p.nbr_off, p.n);
  long long stot = 0;
  if (p.strong) stot = block_scan_counts(p.snbr_cnt, p.snbr_off, p.n);
  if (threadIdx.x == 0) {
    flags->overflow = tot > p.nbr_cap ? 1 : 0;
    // a build that did not classify leaves the strong list unusable until the
    // next build that does (the FP64 kernels then contribute nothing)
    flags->soverflow = p.strong ? (stot > p.scap ? 1 : 0) : 1;
  }
}

// ------------------------------------------------------------ strong pairs
//
// The FP32 pair maths rounds every pair term to ~1e-7 of its size.  In a
// polydisperse system the reference's error scale is the contact force of
// the smallest particles, and near-contact pairs of large particles carry
// terms of ~10-100 such contact forces, so those few pairs (~0.2 % of the
// list at N = 32768, log-normal sigma 0.2) hold most of the FP32 error.  They
// are classified at each list build by the force weight |mu_i| |mu_j| / r^4
// and evaluated in FP64 with the reference's formula
// (src/interaction.cpp:396-417), one thread per entry of the strong list.
// The FP32 passes do this work themselves: the warps of k_real take the
// strong list in chunks of 32 entries, spread evenly over the grid, before
// their own particle, so the FP64 pipe (a small fraction of the FP32 rate on
// GB300, otherwise idle here) works under the FP32 pair loop of the other
// warps.  Each entry's terms go to svals; the integrator adds a particle's
// entries in list order (deterministic).  The FP32 pass keeps the overlap
// push of these pairs; the distance is clamped to contact here too.
// g1(s) = erfc(s) + (2 s / sqrt(pi)) exp(-s^2), the factor of 1/r^3 in the
// pair coefficient a1 (s = alpha r).  From its power series for s <= 1.5:
// g1 = 1 - (4 / sqrt(pi)) s^3 sum_k (-1)^k s^2k / (k! (2k + 3)), 18 terms
// (relative error < 3e-10 at s = 1.5, at the FP64 rounding level below
// s = 1), one branch-free polynomial instead of erfc's range branches;
// beyond, with erfc.  ex = exp(-s^2).
__device__ __forceinline__ double ewald_g1(double s, double ex) {
  const double x = s * s;
  if (x <= 2.25) {
    double q = -7.598533119852758e-17;
    q = fma(q, x, 1.3655649521106815e-15);
    q = fma(q, x, -2.317322342975702e-14);
    q = fma(q, x, 3.7002405153966856e-13);
    q = fma(q, x, -5.537601323041936e-12);
    q = fma(q, x, 7.732132217728926e-11);
    q = fma(q, x, -1.0020843354176688e-09);
    q = fma(q, x, 1.1981443140863431e-08);
    q = fma(q, x, -1.3122532963802806e-07);
    q = fma(q, x, 1.3053467000835422e-06);
    q = fma(q, x, -1.1671335200746965e-05);
    q = fma(q, x, 9.259259259259259e-05);
    q = fma(q, x, -0.000641025641025641);
    q = fma(q, x, 0.003787878787878788);
    q = fma(q, x, -0.018518518518518517);
    q = fma(q, x, 0.07142857142857142);
    q = fma(q, x, -0.2);
    q = fma(q, x, 0.3333333333333333);
    return fma(-2.256758334191025 * s * x, q, 1.0);  // 4 / sqrt(pi)
  }
  return erfc(s) + 1.1283791670955126 * s * ex;  // 2 / sqrt(pi)
}

// The FP64 terms of strong entry (i, j): v[0..2] field, and for FULL
// v[3..5] force, v[6..8] pressure.
template <bool FULL>
__device__ __forceinline__ void strong_entry(const RealParams& p, int2 ij, double v[9]) {
  const float4* gmu = (const float4*)p.s.mu;
  const int4 xi = p.s.xi[ij.x], xj = p.s.xi[ij.y];
  const float4 fi = gmu[ij.x], fj = gmu[ij.y];
  const double sc = 2.3283064365386963e-10;  // 2^-32
  // wrapping differences of the fixed-point coordinates: the exact minimum image
  const double dx = (double)(int)((unsigned)xj.x - (unsigned)xi.x) * sc;
  const double dy = (double)(int)((unsigned)xj.y - (unsigned)xi.y) * sc;
  const double dz = (double)(int)((unsigned)xj.z - (unsigned)xi.z) * sc;
  const double r2 = dx * dx + dy * dy + dz * dz;
  double ire = rsqrt(r2), r = r2 * ire;
  const double ux = dx * ire, uy = dy * ire, uz = dz * ire;
  const double dcont = (double)fi.w + (double)fj.w + p.cont_eps;
  if (r < dcont) {
    r = dcont;
    ire = 1.0 / r;
  }
  const double ire2 = ire * ire, re2 = r * r;
  const double ex = exp(-p.al2 * re2);
  const double t = p.c2a * ex * ire2;
  const double a1 = ewald_g1(p.alpha * r, ex) * ire2 * ire;  // = erfc(alpha r) / r^3 + t
  const double a2 = 3.0 * a1 * ire2 + 2.0 * p.al2 * t;
  double mix = fi.x, miy = fi.y, miz = fi.z, mjx = fj.x, mjy = fj.y, mjz = fj.z;
  if (p.smm) {  // the master moments in FP64 (the sorted view holds them rounded to FP32)
    const int n = p.n, pi = p.s.perm[ij.x], pj = p.s.perm[ij.y];
    const double gi = p.smag[pi], gj = p.smag[pj];
    mix = p.smm[pi] * gi;
    miy = p.smm[n + pi] * gi;
    miz = p.smm[2 * n + pi] * gi;
    mjx = p.smm[pj] * gj;
    mjy = p.smm[n + pj] * gj;
    mjz = p.smm[2 * n + pj] * gj;
  }
  const double d2 = mjx * ux + mjy * uy + mjz * uz;
  const double c1 = a2 * d2 * re2;
  v[0] = c1 * ux - a1 * mjx;
  v[1] = c1 * uy - a1 * mjy;
  v[2] = c1 * uz - a1 * mjz;
  if constexpr (FULL) {
    const double a3 = 5.0 * a2 * ire2 + 4.0 * p.al4 * t;
    const double d1 = mix * ux + miy * uy + miz * uz;
    const double m12 = mix * mjx + miy * mjy + miz * mjz;
    const double s1 = (a2 * m12 - a3 * d1 * d2 * re2) * r;
    const double s2 = a2 * r;
    const double vx = s1 * ux + s2 * (d2 * mix + d1 * mjx);
    const double vy = s1 * uy + s2 * (d2 * miy + d1 * mjy);
    const double vz = s1 * uz + s2 * (d2 * miz + d1 * mjz);
    v[3] = -vx;
    v[4] = -vy;
    v[5] = -vz;
    v[6] = r * ux * vy;
    v[7] = r * ux * vz;
    v[8] = r * uy * vz;
  }
}

// The chunks of the strong list that warp k (one warp per particle) takes:
// with C chunks of 32 entries and n warps, every stride-th warp, stride =
// n / C, takes one chunk (or each warp several when C > n).  A chunk's
// entries are grouped by owner particle (list order); the field and force
// terms are added per owner within the chunk (segmented warp sum, fixed
// order) and stored at the owner's first entry in the chunk, so a particle
// has one partial per chunk it spans.  The pressure, needed only as a total,
// is added over the whole chunk and stored at the chunk's first entry.
template <bool FULL>
__device__ __forceinline__ void strong_chunks(const RealParams& p, int k, int lane) {
  const StepFlags* fl = p.flags;
  if (fl->overflow || fl->soverflow) return;
  const int total = (int)min((long long)p.snbr_off[p.n], p.scap);
  const int chunks = (total + 31) >> 5;
  if (chunks == 0) return;
  const int n = p.n;
  const int stride = max(1, n / chunks);
  if (k % stride) return;
  const int step = (n + stride - 1) / stride;
  const size_t cap = (size_t)p.scap;
  constexpr int NS = FULL ? 6 : 3;  // components summed per owner
  for (int c = k / stride; c < chunks; c += step) {
    const int e = c * 32 + lane;
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int owner = -1 - lane;  // lanes past the end: segments of their own
    if (e < total) {
      const int2 ij = p.snbr[e];
      if ((unsigned)ij.x < (unsigned)n && (unsigned)ij.y < (unsigned)n) {  // always, after a build
        owner = ij.x;
        strong_entry<FULL>(p, ij, v);
      }
    }
    // segmented suffix sums: lane l ends with the sum over [l, end of its run]
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int ow = __shfl_down_sync(kFull, owner, o);
      const bool same = lane + o < 32 && ow == owner;
#pragma unroll
      for (int q = 0; q < NS; q++) {
        const double t = __shfl_down_sync(kFull, v[q], o);
        if (same) v[q] += t;
      }
    }
    const int prev = __shfl_up_sync(kFull, owner, 1);
    if (e < total && (lane == 0 || prev != owner)) {
#pragma unroll
      for (int q = 0; q < NS; q++) p.svals[q * cap + e] = v[q];
    }
    if constexpr (FULL) {
#pragma unroll
      for (int q = 6; q < 9; q++) {
        const double t = warp_sum(v[q]);
        if (lane == 0) p.svals[q * cap + e] = t;
      }
    }
  }
}

// ------------------------------------------------------------ evaluation

template <typename T, bool FULL, bool COAT, int NW = kRealWarps>
__device__ __forceinline__ void real_eval(const RealParams& p, int bx) {
  using T4 = typename V4<T>::t;
  constexpr bool F32 = std::is_same<T, float>::value;
  __shared__ float4 q[NW][64];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = bx * NW + wib;
  if (k >= p.n) return;  // whole warp; no block-level synchronisation below
  if constexpr (F32 && !COAT) {
    if (p.strong && !p.flags->overflow) strong_chunks<FULL>(p, k, lane);
  }
  Acc<T> a;
  Acc2 a2;  // packed sums (mixed path list loop)
  const T4 mi = ((const T4*)p.s.mu)[k];
  const Self<T> me = load_self<T, COAT>(p, k);
  const float rc2_fix = p.pk.rc2f;  // (rc / (L 2^-32))^2
  const float wdc = (float)mi.w + p.pk.eps;  // own core radius + contact offset

  // pair terms with the neighbour's loaded coordinates and moment (mixed path)
  auto eval_loaded = [&](const int4& sj, const T4& mj) {
    if constexpr (F32) {
      // wrapping 32-bit differences are the exact minimum image
      const float dxf = (float)(sj.x - me.si.x), dyf = (float)(sj.y - me.si.y), dzf = (float)(sj.z - me.si.z);
      if (dxf * dxf + dyf * dyf + dzf * dzf < rc2_fix) {
        const float sc = 2.3283064365386963e-10f;  // 2^-32
        const float dx = dxf * sc, dy = dyf * sc, dz = dzf * sc;
        pair_terms<T, FULL, COAT>(p, dx, dy, dz, dx * dx + dy * dy + dz * dz, mi, mj, me.oi, COAT ? sj.w : 0, a);
      }
    }
  };
  // pair vector from i to sorted particle j, and the in-range test
  auto eval = [&](int j) {
    const T4 mj = ((const T4*)p.s.mu)[j];
    if constexpr (F32) {
      const int4 sj = p.s.xi[j];
      const float dxf = (float)(sj.x - me.si.x), dyf = (float)(sj.y - me.si.y), dzf = (float)(sj.z - me.si.z);
      if (dxf * dxf + dyf * dyf + dzf * dzf < rc2_fix) {
        const float sc = 2.3283064365386963e-10f;
        const float dx = dxf * sc, dy = dyf * sc, dz = dzf * sc;
        pair_terms<T, FULL, COAT>(p, dx, dy, dz, dx * dx + dy * dy + dz * dz, mi, mj, me.oi, COAT ? sj.w : 0, a);
      }
    } else {
      const double4_32a dj = p.s.xd[j];
      double dx = dj.x - me.di.x, dy = dj.y - me.di.y, dz = dj.z - me.di.z;
      dx -= (double)(dx > 0.5);
      dx += (double)(dx < -0.5);
      dy -= (double)(dy > 0.5);
      dy += (double)(dy < -0.5);
      dz -= (double)(dz > 0.5);
      dz += (double)(dz < -0.5);
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < p.rc2) pair_terms<T, FULL, COAT>(p, dx, dy, dz, r2, mi, mj, me.oi, COAT ? p.s.perm[j] : 0, a);
    }
  };

  if (!p.flags->overflow) {
    // Verlet list of this particle
    const int* lst = p.nbr + p.nbr_off[k];
    const int cnt = p.nbr_off[k + 1] - p.nbr_off[k];
    if constexpr (F32) {
      // two batches of 32 entries per iteration, all gathers issued first;
      // the list indices of the next iteration are loaded one ahead, so a
      // gather waits on one memory round trip instead of two
      // entries with the sign bit set are strong pairs (FP64 kernels) when
      // the context evaluates them there, ordinary ones otherwise
      const int sflag = p.strong ? (int)0x80000000u : 0;
      // the list is streamed once per pass: evict-first loads leave L1 to the
      // neighbour gathers (0.3-0.9 % per step)
      int ja_n = lane < cnt ? __ldcs(lst + lane) : k, jb_n = 32 + lane < cnt ? __ldcs(lst + 32 + lane) : k;
      for (int t0 = 0; t0 < cnt; t0 += 64) {
        const int ta = t0 + lane, tb = t0 + 32 + lane;
        const bool va = ta < cnt, vb = tb < cnt;
        const bool sta = (ja_n & sflag) != 0, stb = (jb_n & sflag) != 0;
        const int ja = ja_n & 0x7fffffff, jb = jb_n & 0x7fffffff;
        ja_n = ta + 64 < cnt ? __ldcs(lst + ta + 64) : k;
        jb_n = tb + 64 < cnt ? __ldcs(lst + tb + 64) : k;
        const int4 sa = p.s.xi[ja], sb = p.s.xi[jb];
        const T4 ma = ((const T4*)p.s.mu)[ja], mb = ((const T4*)p.s.mu)[jb];
        if constexpr (!COAT) {
          // both neighbours in the halves of packed FP32 operations (the
          // field + force pass assembles each pair in scalar code)
          const float2 dxf = pk((float)(sa.x - me.si.x), (float)(sb.x - me.si.x));
          const float2 dyf = pk((float)(sa.y - me.si.y), (float)(sb.y - me.si.y));
          const float2 dzf = pk((float)(sa.z - me.si.z), (float)(sb.z - me.si.z));
          const float2 r2f = fma2(dzf, dzf, fma2(dyf, dyf, mul2(dxf, dxf)));
          const bool inA = va && r2f.x < rc2_fix, inB = vb && r2f.y < rc2_fix;
          // unconditional: nearly every iteration has a pair in range, and
          // entries out of range carry weight 0
          pair_terms2<FULL>(p.pk, wdc, dxf, dyf, dzf, r2f, inA, inB, inA && !sta, inB && !stb, rc2_fix, mi, ma,
                            mb, a, a2);
        } else {
          if (va) eval_loaded(sa, ma);
          if (vb) eval_loaded(sb, mb);
        }
      }
    } else {
      int jn = lane < cnt ? lst[lane] : 0;
      for (int t0 = 0; t0 < cnt; t0 += 32) {
        const int j = jn & 0x7fffffff;
        const bool valid = t0 + lane < cnt;
        if (t0 + 32 + lane < cnt) jn = lst[t0 + 32 + lane];
        if (valid) eval(j);
      }
    }
  } else {
    // fallback: scan the cells; in-range candidates through the warp queue
    int head = 0, tail = 0;
    auto flush = [&](int cnt) {
      __syncwarp();
      const float4 e = lane < cnt ? q[wib][(head + lane) & 63] : make_float4(0, 0, 0, 0);
      __syncwarp();
      head += cnt;
      if (lane < cnt) eval(__float_as_int(e.w));
    };
    scan_rows<T>(p, k, lane, me, p.rc2, [&](bool in, int j, float, float, float) {
      const unsigned mask = __ballot_sync(kFull, in);
      if (in) q[wib][(tail + __popc(mask & lanemask_lt())) & 63] = make_float4(0, 0, 0, __int_as_float(j));
      tail += __popc(mask);
      if (tail - head >= 32) flush(32);
    });
    if (tail - head > 0) flush(tail - head);
  }

  if constexpr (F32 && !FULL && !COAT) {
    a.b0 += a2.b0.x + a2.b0.y;
    a.b1 += a2.b1.x + a2.b1.y;
    a.b2 += a2.b2.x + a2.b2.y;
  }
  a.b0 = warp_sum(a.b0);
  a.b1 = warp_sum(a.b1);
  a.b2 = warp_sum(a.b2);
  if constexpr (FULL) {
    a.f0 = warp_sum(a.f0);
    a.f1 = warp_sum(a.f1);
    a.f2 = warp_sum(a.f2);
    a.o0 = warp_sum(a.o0);
    a.o1 = warp_sum(a.o1);
    a.o2 = warp_sum(a.o2);
    a.p0 = warp_sum(a.p0);
    a.p1 = warp_sum(a.p1);
    a.p2 = warp_sum(a.p2);
    a.np = warp_sum(a.np);
  }
  if (lane == 0) {
    T* B = (T*)p.B;
    const int n = p.n;
    B[k] = a.b0;
    B[n + k] = a.b1;
    B[2 * n + k] = a.b2;
    if constexpr (FULL) {
      T* F = (T*)p.F;
      T* O = (T*)p.ov;
      F[k] = a.f0;
      F[n + k] = a.f1;
      F[2 * n + k] = a.f2;
      O[k] = a.o0;
      O[n + k] = a.o1;
      O[2 * n + k] = a.o2;
      p.Ppart[3 * k] = (double)a.p0;
      p.Ppart[3 * k + 1] = (double)a.p1;
      p.Ppart[3 * k + 2] = (double)a.p2;
      if (p.npairs) atomicAdd(p.npairs, (unsigned long long)a.np);
    }
  }
}

static int num_sms() {
  // initialised once (thread-safe: contexts may be created on several threads)
  static const int nsm = [] {
    int dev = 0, k = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&k, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || k <= 0) k = 148;
    return k;
  }();
  return nsm;
}


// ------------------------------------------------------------ entry points

// Grid-stride over the particle blocks: most steps do not rebuild, and a
// grid of a few blocks per SM then costs one flag read per block.
template <typename T, bool FILL>
__global__ void __launch_bounds__(kRealWarps * 32) k_nbr_build(RealParams p, int nblk) {
  if (!p.flags->rebuild) return;
  for (int bx = blockIdx.x; bx < nblk; bx += gridDim.x) nbr_build<T, FILL>(p, bx);
}
__global__ void __launch_bounds__(1024) k_nbr_scan(RealParams p) { nbr_scan(p); }
// The FP32 passes without coating keep the occupancy of their pair loops
// (field: 9 blocks of 4 warps per SM, 56 registers; field + force: 7 blocks,
// 72 registers): the FP64 strong-pair code in the same kernel must not
// raise the register count.
template <typename T, bool FULL, bool COAT>
__global__ void __launch_bounds__(((FULL && COAT) ? kRealWarps : kFieldWarps) * 32,
                                  (std::is_same<T, float>::value && !COAT) ? (FULL ? 7 : 9) : 1) k_real(RealParams p) {
  real_eval<T, FULL, COAT, (FULL && COAT) ? kRealWarps : kFieldWarps>(p, blockIdx.x);
}

// persistent: blocks stride over the task table (see md_cells.cu); the
// list build and the pair loop are warp-private (no block barrier)
template <bool FILL>
__global__ void __launch_bounds__(kRealWarps * 32) k_nbr_build_packed(const RealParams* __restrict__ ps,
                                                                      const Task* __restrict__ tk, int ntask, WorkQ* wq,
                                                                      const unsigned* anyrb) {
  if (!__ldcg(anyrb)) return;  // the whole grid: no system rebuilds this step
  for_tasks<false>(tk, ntask, wq, [&](const Task& t) {
      nbr_build<float, FILL>(ps[t.rep], t.blk);
  });
}
__global__ void __launch_bounds__(1024) k_nbr_scan_packed(const RealParams* __restrict__ ps) {
  const RealParams p = ps[blockIdx.x];
  nbr_scan(p);
}
// the block shape of the single-system passes (k_real): 8 warps with
// coating in the field + force pass, otherwise 4; 6 (field + force) or 7
// (field) blocks per SM, one fewer than k_real's 7 / 9: the task loop
// around the pair loop needs the registers (at 7 / 9 both spilled, and the
// field sweep ran 1.1 % slower)
template <bool FULL, bool COAT>
__global__ void __launch_bounds__(((FULL && COAT) ? kRealWarps : kFieldWarps) * 32, COAT ? 2 : (FULL ? 6 : 7))
    k_real_packed(const RealParams* __restrict__ ps, const Task* __restrict__ tk, int ntask, WorkQ* wq) {
  for_tasks<false>(tk, ntask, wq, [&](const Task& t) {
      real_eval<float, FULL, COAT, (FULL && COAT) ? kRealWarps : kFieldWarps>(ps[t.rep], t.blk);
  });
}

int real_blocks(int n) { return (n + kRealWarps - 1) / kRealWarps; }
int real_pass_blocks(int n) { return (n + kFieldWarps - 1) / kFieldWarps; }

int launch_nbr(cudaStream_t st, const RealParams& p, StepFlags* flags, bool fp64) {
  const int nsm = num_sms();
  const int nblk = real_blocks(p.n);
  dim3 grid(std::min(nblk, 8 * nsm)), block(kRealWarps * 32);
  if (fp64)
    k_nbr_build<double, false><<<grid, block, 0, st>>>(p, nblk);
  else
    k_nbr_build<float, false><<<grid, block, 0, st>>>(p, nblk);
  (void)flags;
  k_nbr_scan<<<1, 1024, 0, st>>>(p);
  if (fp64)
    k_nbr_build<double, true><<<grid, block, 0, st>>>(p, nblk);
  else
    k_nbr_build<float, true><<<grid, block, 0, st>>>(p, nblk);
  return 3;
}

int launch_real(cudaStream_t st, const RealParams& p, bool full, bool fp64) {
  const int nw = (full && p.coat) ? kRealWarps : kFieldWarps;
  dim3 grid((p.n + nw - 1) / nw), block(nw * 32);
  if (fp64) {
    if (full)
      p.coat ? k_real<double, true, true><<<grid, block, 0, st>>>(p)
             : k_real<double, true, false><<<grid, block, 0, st>>>(p);
    else
      k_real<double, false, false><<<grid, block, 0, st>>>(p);
  } else {
    if (full)
      p.coat ? k_real<float, true, true><<<grid, block, 0, st>>>(p)
             : k_real<float, true, false><<<grid, block, 0, st>>>(p);
    else
      k_real<float, false, false><<<grid, block, 0, st>>>(p);
  }
  return 1;
}

int launch_nbr_packed(cudaStream_t st, const RealParams* ps, int R, const Packed& real, const unsigned* anyrb) {
  const int th = kRealWarps * 32;
  if (real.n)
    k_nbr_build_packed<false><<<persistent_grid((const void*)k_nbr_build_packed<false>, th, 0, real.n), th, 0, st>>>(
        ps, real.tasks, real.n, real.wq, anyrb);
  k_nbr_scan_packed<<<R, 1024, 0, st>>>(ps);
  if (real.n)
    k_nbr_build_packed<true><<<persistent_grid((const void*)k_nbr_build_packed<true>, th, 0, real.n), th, 0, st>>>(
        ps, real.tasks, real.n, real.wq, anyrb);
  return 3;
}

int launch_real_packed(cudaStream_t st, const RealParams* ps, const Packed& real, const Packed& pass, bool full,
                       bool coat) {
  auto go = [&](auto kern, const Packed& tb, int th) {
    kern<<<persistent_grid((const void*)kern, th, 0, tb.n), th, 0, st>>>(ps, tb.tasks, tb.n, tb.wq);
  };
  if (full && coat) {
    if (!real.n) return 0;
    go(k_real_packed<true, true>, real, kRealWarps * 32);
  } else {
    if (!pass.n) return 0;
    full ? go(k_real_packed<true, false>, pass, kFieldWarps * 32) : go(k_real_packed<false, false>, pass, kFieldWarps * 32);
  }
  return 1;
}

}  // namespace md
