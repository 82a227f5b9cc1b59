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
// Mapping: one warp per (cell-sorted) particle i.  The warp walks the rows of
// its cell stencil; lane r first computes row r's cell range, culled to the
// cells that intersect the cutoff sphere around i.  Lanes then test 32
// candidates at a time (the next 32 are prefetched), and the in-range ones
// are compacted with a ballot into a per-warp queue in shared memory that
// holds the pair vector.  The pair maths (erfc, exp, ~90 flops) runs only on
// full 32-pair batches, so every lane does useful work.  Per-lane sums are
// reduced with warp shuffles; each warp writes its own pressure partial.
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
#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kRealWarps = 8;  // warps (particles) per block

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
  T ir0, ux, uy, uz, r, ire;
  if constexpr (std::is_same<T, float>::value) {
    ir0 = rsqrtf(r2);
  } else {
    ir0 = rsqrt(r2);
  }
  const T r0 = r2 * ir0;
  ux = dx * ir0;
  uy = dy * ir0;
  uz = dz * ir0;
  r = r0;
  ire = ir0;
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

template <typename T, bool FULL, bool COAT>
__global__ void __launch_bounds__(kRealWarps * 32) k_real(RealParams p) {
  using T4 = typename V4<T>::t;
  constexpr bool F32 = std::is_same<T, float>::value;
  __shared__ float4 q[kRealWarps][64];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kRealWarps + wib;
  if (k >= p.n) return;  // whole warp; no block-level synchronisation below
  Acc<T> a;
  const T4 mi = ((const T4*)p.s.mu)[k];
  int4 si = make_int4(0, 0, 0, 0);
  double4_32a di = make_double4_32a(0, 0, 0, 0);
  float xix, xiy, xiz;
  int oi;
  if constexpr (F32) {
    si = p.s.xi[k];
    const float sc = 2.3283064365386963e-10f;
    xix = (float)si.x * sc;
    xiy = (float)si.y * sc;
    xiz = (float)si.z * sc;
    oi = si.w;
  } else {
    di = p.s.xd[k];
    const float4 f = p.s.xf[k];
    xix = f.x;
    xiy = f.y;
    xiz = f.z;
    oi = COAT ? p.s.perm[k] : 0;
  }
  const int ncx = p.grid.ncx, m = p.grid.reach, side = 2 * m + 1, R = side * side;
  const int cell = p.s.cell[k];
  const int cx = cell % ncx, cy = (cell / ncx) % ncx, cz = cell / (ncx * ncx);
  const float inv = 1.0f / (float)ncx;
  const float rct2 = (float)p.rc2_test;
  // fixed-point cutoff: r^2 in units of (L / 2^32)^2
  const float rc2_fix = (float)(p.rc2 * 18446744073709551616.0);
  const int* cs = p.s.cell_start;
  int head = 0, tail = 0;

  auto flush = [&](int cnt) {
    __syncwarp();
    float4 e = lane < cnt ? q[wib][(head + lane) & 63] : make_float4(0, 0, 0, 0);
    __syncwarp();
    head += cnt;
    if (lane < cnt) {
      const int j = __float_as_int(e.w);
      const T4 mj = ((const T4*)p.s.mu)[j];
      int oj = 0;
      if constexpr (COAT) oj = F32 ? p.s.xi[j].w : p.s.perm[j];
      if constexpr (F32) {
        pair_terms<T, FULL, COAT>(p, e.x, e.y, e.z, e.x * e.x + e.y * e.y + e.z * e.z, mi, mj, oi, oj, a);
      } else {
        const double4_32a dj = p.s.xd[j];
        double dx = dj.x - di.x, dy = dj.y - di.y, dz = dj.z - di.z;
        dx -= (double)(dx > 0.5);
        dx += (double)(dx < -0.5);
        dy -= (double)(dy > 0.5);
        dy += (double)(dy < -0.5);
        dz -= (double)(dz > 0.5);
        dz += (double)(dz < -0.5);
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < p.rc2) pair_terms<T, FULL, COAT>(p, dx, dy, dz, r2, mi, mj, oi, oj, a);
      }
    }
  };
  auto enqueue = [&](bool in, float4 v) {
    const unsigned mask = __ballot_sync(kFull, in);
    if (in) q[wib][(tail + __popc(mask & lanemask_lt())) & 63] = v;
    tail += __popc(mask);
    if (tail - head >= 32) flush(32);
  };
  auto scan = [&](int s, int e) {
    if (s >= e) return;
    if constexpr (F32) {
      const float sc = 2.3283064365386963e-10f;
      int4 nxt = s + lane < e ? p.s.xi[s + lane] : make_int4(0, 0, 0, 0);
      for (int j0 = s; j0 < e; j0 += 32) {
        const int j = j0 + lane;
        const int4 sj = nxt;
        if (j0 + 32 + lane < e) nxt = p.s.xi[j0 + 32 + lane];
        const float dx = (float)(sj.x - si.x), dy = (float)(sj.y - si.y), dz = (float)(sj.z - si.z);
        const bool in = j < e && j != k && dx * dx + dy * dy + dz * dz < rc2_fix;
        enqueue(in, make_float4(dx * sc, dy * sc, dz * sc, __int_as_float(j)));
      }
    } else {
      float4 nxt = s + lane < e ? p.s.xf[s + lane] : make_float4(0, 0, 0, 0);
      for (int j0 = s; j0 < e; j0 += 32) {
        const int j = j0 + lane;
        const float4 xj = nxt;
        if (j0 + 32 + lane < e) nxt = p.s.xf[j0 + 32 + lane];
        float dx = xj.x - xix, dy = xj.y - xiy, dz = xj.z - xiz;
        dx -= rintf(dx);
        dy -= rintf(dy);
        dz -= rintf(dz);
        const bool in = j < e && j != k && dx * dx + dy * dy + dz * dz < rct2;
        enqueue(in, make_float4(0, 0, 0, __int_as_float(j)));
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
        const float ey = fmaxf(0.f, fmaxf(ylo - xiy, xiy - yhi));
        const float ez = fmaxf(0.f, fmaxf(zlo - xiz, xiz - zhi));
        const float d2 = ey * ey + ez * ez;
        ok = d2 < rct2;
        if (ok) {
          const float w = sqrtf(rct2 - d2);
          xlo = max(xlo, (int)floorf((xix - w + 0.5f) * ncx));
          xhi = min(xhi, (int)floorf((xix + w + 0.5f) * ncx));
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
    for (int rr = 0; rr < nr; rr++) {
      const int s0 = __shfl_sync(kFull, a0, rr), e0 = __shfl_sync(kFull, b0, rr);
      const int s1 = __shfl_sync(kFull, a1, rr), e1 = __shfl_sync(kFull, b1, rr);
      scan(s0, e0);
      scan(s1, e1);
    }
  }
  if (tail - head > 0) flush(tail - head);

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

int real_blocks(int n) { return (n + kRealWarps - 1) / kRealWarps; }

int launch_real(cudaStream_t st, const RealParams& p, bool full, bool fp64) {
  dim3 grid(real_blocks(p.n)), block(kRealWarps * 32);
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

}  // namespace md
