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
// candidates at a time against rc (float coordinates, minimum image), and the
// in-range candidates are compacted with a ballot into a per-warp queue in
// shared memory.  The pair maths (erfc, exp, ~90 flops) runs only on full
// 32-pair batches, so every lane does useful work.  Per-lane sums are
// reduced with warp shuffles at the end.
//
// Geometry precision (mixed path): the pair vector comes from 32-bit
// fixed-point coordinates, whose wrapping subtraction is the exact minimum
// image; FP32 conversion then gives ~6e-8 relative error in r at any
// distance.  The FP64 path uses FP64 box coordinates and the reference's
// fold (d > L/2 -> d - L, d < -L/2 -> d + L).
//
// Overlap push: CompInteractVecs moves cores apart in place while it walks
// the pairs, so later pairs see moved positions.  Here every overlap is
// resolved from the same starting positions (Jacobi): particle i collects
// -1/2 (dCont - r) r_hat_ij over its overlapping neighbours, r is clamped to
// dCont for the Ewald terms, and the displacement is applied with the
// translation step.  For configurations without overlaps the two agree.
//
// Roofline: FP32/SFU issue bound.  Algorithmic FLOPs per in-range pair
// (counted from the reference formula): 86 full, 46 field only.
#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kRealWarps = 8;  // warps (particles) per block

__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }
__device__ __forceinline__ float ex(float x) { return expf(x); }
__device__ __forceinline__ double ex(double x) { return exp(x); }
__device__ __forceinline__ float erc(float x) { return erfcf(x); }
__device__ __forceinline__ double erc(double x) { return erfc(x); }

template <typename T>
struct Acc {
  T b0 = 0, b1 = 0, b2 = 0, f0 = 0, f1 = 0, f2 = 0, o0 = 0, o1 = 0, o2 = 0, p0 = 0, p1 = 0, p2 = 0;
  int np = 0;  // in-range pairs seen by this lane
};

template <typename T, bool FULL, bool COAT>
__device__ __forceinline__ void pair_math(const RealParams& p, int j, int k, const int4& si, const double4_32a& di,
                                          const typename V4<T>::t& mi, Acc<T>& a) {
  using T4 = typename V4<T>::t;
  T dx, dy, dz;
  int4 sj;
  if constexpr (std::is_same<T, float>::value) {
    sj = p.s.xi[j];
    const float q = 2.3283064365386963e-10f;  // 2^-32
    dx = (float)(sj.x - si.x) * q;
    dy = (float)(sj.y - si.y) * q;
    dz = (float)(sj.z - si.z) * q;
  } else {
    double4_32a dj = p.s.xd[j];
    dx = dj.x - di.x;
    dy = dj.y - di.y;
    dz = dj.z - di.z;
    dx -= (double)(dx > 0.5);
    dx += (double)(dx < -0.5);
    dy -= (double)(dy > 0.5);
    dy += (double)(dy < -0.5);
    dz -= (double)(dz > 0.5);
    dz += (double)(dz < -0.5);
  }
  const T r2 = dx * dx + dy * dy + dz * dz;
  if (!(r2 < (T)p.rc2)) return;
  a.np++;
  const T4 mj = ((const T4*)p.s.mu)[j];
  const T ir0 = rsq(r2);
  const T r0 = r2 * ir0;
  const T ux = dx * ir0, uy = dy * ir0, uz = dz * ir0;
  T r = r0;
  const T dcont = mi.w + mj.w + (T)p.cont_eps;
  if (r < dcont) {
    if constexpr (FULL) {
      const T h = (T)0.5 * (dcont - r);
      a.o0 -= h * ux;
      a.o1 -= h * uy;
      a.o2 -= h * uz;
    }
    r = dcont;
  }
  const T ire = (T)1 / r;
  const T ire2 = ire * ire;
  const T re2 = r * r;
  const T e = ex(-(T)p.al2 * re2);
  const T t = (T)p.c2a * e * ire2;
  const T a1 = erc((T)p.alpha * r) * ire2 * ire + t;
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
        int oi, oj;
        double rd;
        if constexpr (std::is_same<T, float>::value) {
          oi = si.w;
          oj = sj.w;
          const double q = 2.3283064365386963e-10;
          double ddx = (double)(sj.x - si.x) * q, ddy = (double)(sj.y - si.y) * q, ddz = (double)(sj.z - si.z) * q;
          rd = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
        } else {
          oi = p.s.perm[k];
          oj = p.s.perm[j];
          rd = (double)r0;
        }
        const double ri = p.rMag_u[oi], rj = p.rMag_u[oj];
        double dc = ri + rj + p.cont_eps;
        if (rd < dc) rd = dc;
        // steric repulsion is asymmetric: dDelta and the prefactor use the
        // pair's lower particle index as "idx1" (interaction.cpp:768-775)
        double ra = oi < oj ? ri : rj, rb = oi < oj ? rj : ri;
        double dDelta = 2.0 * (ra + p.eff_len);
        double s = rd <= dDelta ? (2.0 * rb / (ra + rb)) * p.ster * ra * ra * log(dDelta / rd) : 0.0;
        s += (ri * rj / (ri + rj)) * p.elec * exp(-p.kappa * (rd - ri - rj));
        double g1 = (rd - ri - rj) * (rd + ri + rj), g2 = rd * rd - (ri - rj) * (ri - rj);
        double c4 = 4.0 * ri * rj;
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
  __shared__ int q[kRealWarps][64];
  __shared__ double psh[kRealWarps][3];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kRealWarps + wib;
  const bool active = k < p.n;
  Acc<T> a;
  if (active) {
    const float4 xi = p.s.xf[k];
    const T4 mi = ((const T4*)p.s.mu)[k];
    int4 si = make_int4(0, 0, 0, 0);
    double4_32a di = make_double4_32a(0, 0, 0, 0);
    if constexpr (std::is_same<T, float>::value)
      si = p.s.xi[k];
    else
      di = p.s.xd[k];
    const int ncx = p.grid.ncx, m = p.grid.reach, side = 2 * m + 1, R = side * side;
    const int cell = p.s.cell[k];
    const int cx = cell % ncx, cy = (cell / ncx) % ncx, cz = cell / (ncx * ncx);
    const float inv = 1.0f / (float)ncx;
    const float rct2 = (float)p.rc2_test;
    const int* cs = p.s.cell_start;
    int head = 0, tail = 0;

    auto flush = [&](int cnt) {
      __syncwarp();
      int jj = lane < cnt ? q[wib][(head + lane) & 63] : -1;
      __syncwarp();
      head += cnt;
      if (jj >= 0) pair_math<T, FULL, COAT>(p, jj, k, si, di, mi, a);
    };
    auto scan = [&](int s, int e) {
      for (int j0 = s; j0 < e; j0 += 32) {
        const int j = j0 + lane;
        bool in = false;
        if (j < e && j != k) {
          const float4 xj = p.s.xf[j];
          float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
          dx -= rintf(dx);
          dy -= rintf(dy);
          dz -= rintf(dz);
          in = dx * dx + dy * dy + dz * dz < rct2;
        }
        const unsigned mask = __ballot_sync(kFull, in);
        if (in) q[wib][(tail + __popc(mask & lanemask_lt())) & 63] = j;
        tail += __popc(mask);
        if (tail - head >= 32) flush(32);
      }
    };

    for (int rb = 0; rb < R; rb += 32) {
      const int r = rb + lane;
      int a0 = 0, b0 = 0, a1 = 0, b1 = 0;
      if (r < R) {
        const int dy = r % side - m, dz = r / side - m;
        const int uy = cy + dy, uz = cz + dz;
        float d2 = 0.f;
        int xlo = cx - m, xhi = cx + m;
        bool ok = true;
        if (ncx > 1) {
          const float ylo = uy * inv - 0.5f, yhi = ylo + inv, zlo = uz * inv - 0.5f, zhi = zlo + inv;
          const float ey = fmaxf(0.f, fmaxf(ylo - xi.y, xi.y - yhi));
          const float ez = fmaxf(0.f, fmaxf(zlo - xi.z, xi.z - zhi));
          d2 = ey * ey + ez * ez;
          ok = d2 < rct2;
          if (ok) {
            const float w = sqrtf(rct2 - d2);
            xlo = max(xlo, (int)floorf((xi.x - w + 0.5f) * ncx));
            xhi = min(xhi, (int)floorf((xi.x + w + 0.5f) * ncx));
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
      if (lane == 0 && p.npairs) atomicAdd(p.npairs, (unsigned long long)a.np);
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
      }
    }
  }
  if constexpr (FULL) {
    if (lane == 0) {
      psh[wib][0] = active ? (double)a.p0 : 0.0;
      psh[wib][1] = active ? (double)a.p1 : 0.0;
      psh[wib][2] = active ? (double)a.p2 : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      double s = 0;
      for (int w = 0; w < kRealWarps; w++) s += psh[w][threadIdx.x];
      p.Ppart[3 * blockIdx.x + threadIdx.x] = s;
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
