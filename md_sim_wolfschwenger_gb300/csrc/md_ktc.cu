// md_ktc.cu -- kernel (c) on the tensor cores (mixed path): the
// reciprocal-space Ewald sums of CompDipInteractEwaldF / CompDipFieldEwaldF
// (src/interaction.cpp:429-514, 588-672), the same sums as md_kspace.cu,
// written as complex matrix products over rows of k vectors.
//
// A k row r = (ny, nz) holds n = (nx, ny, nz), nx in [-kc, kc] (column
// q = nx + kc).  With the per-particle phases X_j(nx) = exp(2 pi i nx x_j),
// P_j(r) = Y_j(ny) Z_j(nz):
//   S(n) = sum_j (n . mu_j) X_j(nx) P_j(r) = C_U(r, nx) + nx C_V(r, nx),
//   C_U(r, nx) = sum_j U_j(r) X_j(nx),  U_j(r) = (ny mu_yj + nz mu_zj) P_j(r),
//   C_V(r, nx) = sum_j V_j(r) X_j(nx),  V_j(r) = mu_xj P_j(r),
// a product [rows x particles] x [particles x nx].  The scatter, with
// W_p(r, nx) = nx^p conj(e(n) S(n)) and Q_p(i, r) = sum_nx X_i(nx) W_p(r, nx)
// (a product [particles x nx] x [nx x rows]), is
//   B_i = -cflux sum_r (Re(P Q_1), ny Re(P Q_0), nz Re(P Q_0))
//   F_i = cforce sum_r (mu_x Im(P Q_2) + c Im(P Q_1), ny g, nz g),
//   g = mu_x Im(P Q_1) + c Im(P Q_0),  c = ny mu_y + nz mu_z,  P = P_i(r),
// which the scatter kernel evaluates in the epilogue of its matrix product,
// from the accumulators in tensor memory.  Complex products run as real
// ones: [Re a, Im a] against [[Re b, Im b], [-Im b, Re b]] blocks.
//
// Precision: each FP32 operand is split into TF32 hi + lo and the products
// are hi*hi + hi*lo + lo*hi (three kind::tf32 MMAs into one FP32
// accumulator), ~22 significant bits per product like FP32 arithmetic.  The
// structure factor accumulates chunks of <= 1024 particles in the tensor
// core's FP32 and sums the chunks in FP64 in a fixed order; the scatter sums
// over the nx of a row in the MMA (<= 2 kc + 1 terms), over the rows of a
// tile in FP32 and over tiles with compensated FP32 sums.  All sums have a
// fixed order: results are deterministic.
//
// Kernels:
//   k_sf_tc      grid (M tiles, chunks), 256 threads: generates U, V (A) and
//                X (B) operands of 16 particles per stage in shared memory
//                (two stages: the next is generated while the tensor cores
//                multiply the current one), one thread issues the MMAs;
//                D (128 x NS FP32) lives in tensor memory and is written to
//                chunk partials at the end.
//   k_sf_tc_reduce  FP64 sum of the chunk partials, S(n) = C_U + nx C_V,
//                e(n) S(n), and the scatter's W operand image (hi, lo) in
//                the shared-memory layout the scatter copies in bulk.
//   k_kscat_tc   128 particles per block: the particles' X phases (A) stay in
//                shared memory, W tiles of 64 columns stream in by bulk copy
//                (2-3 stages), two tensor-memory accumulators alternate so
//                the epilogue of one tile overlaps the MMAs of the next.
#include "md_common.cuh"
#include "md_kernels.h"
#include "md_tc.cuh"

#include <algorithm>

namespace md {

constexpr int kSfSC = 16;            // particles per structure-factor stage
constexpr int kSfSK = 2 * kSfSC;     // K elements per stage
constexpr int kSfThreads = 256;
constexpr int kTcMaxKc = 25;         // shared-memory bound of the scatter (two stages)
constexpr int kSfTabPer = (3 * (kTcMaxKc + 1) * kSfSC + kSfThreads - 1) / kSfThreads;  // table entries per thread
constexpr int kScEpiWarps = 8;       // scatter: 2 warps per tensor-memory lane quarter (tile halves)
constexpr int kScThreads = 32 * (kScEpiWarps + 1);  // + one producer warp (bulk copies, MMAs)
constexpr int kScParticles = 128;    // particles per scatter block (tensor-memory lanes)
constexpr int kScCols = 64;          // scatter tile: 64 output columns
constexpr int kScMaxStages = 3;
constexpr size_t kSmemLimit = 227 * 1024 - 5 * 1024;  // dynamic shared memory per block (static <= 4 KB)

// Scatter tile: 64 real columns in two halves of 16 complex columns; a
// half holds RH k rows x P complex columns Q_0 .. Q_{P-1} (+ padding), so
// each half is one 32-column tensor-memory load of an epilogue warp.
template <bool FULL>
struct ScatLayout {
  static constexpr int P = FULL ? 3 : 2;       // Q_p per row
  static constexpr int RH = FULL ? 5 : 8;      // rows per half tile
  static constexpr int RT = 2 * RH;            // rows per tile
  // complex column of Q_p of the tile's row sl
  __host__ __device__ static constexpr int ccol(int sl, int pp) { return (sl / RH) * 16 + (sl % RH) * P + pp; }
};

static int tc_ns(int kc) { return (2 * (2 * kc + 1) + 15) / 16 * 16; }
static int tc_kp(int kc) { return (2 * (2 * kc + 1) + 7) / 8 * 8; }

static size_t sf_smem(int kc) {
  const int ns = tc_ns(kc), k1 = kc + 1;
  const size_t stage = 2 * (size_t)128 * kSfSK * 4 + 2 * (size_t)ns * kSfSK * 4;
  return 2 * stage + (size_t)kSfSC * (3 * k1 + 1) * 8 + (size_t)kSfSC * 16;
}
static size_t scat_smem(int kc, int nst) {
  const int kp = tc_kp(kc);
  return 2 * (size_t)128 * kp * 4 + (size_t)nst * 2 * kScCols * kp * 4;
}

// ------------------------------------------------------ structure factor

__global__ void __launch_bounds__(kSfThreads) k_sf_tc(KParams p) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ double red[3][kSfThreads / 32];
  const int mtile = blockIdx.x, chunk = blockIdx.y;
  const int NS = p.tc_ns, kc = p.kc, K1 = kc + 1, n = p.n;
  const int abytes = 128 * kSfSK * 4, bbytes = NS * kSfSK * 4, sbytes = 2 * abytes + 2 * bbytes;
  const int tstride = 3 * K1 + 1;
  float2* tabs = (float2*)(smem + 2 * sbytes);              // [kSfSC][3 K1 + 1]: X, Y, Z
  float4* mus = (float4*)(tabs + kSfSC * tstride);          // [kSfSC]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p0 = chunk * p.tc_chunk, p1 = min(n, p0 + p.tc_chunk);
  const int nstage = p1 > p0 ? (p1 - p0 + kSfSC - 1) / kSfSC : 0;
  const uint32_t ncols = NS <= 32 ? 32 : (NS <= 64 ? 64 : (NS <= 128 ? 128 : 256));
  const float2* gtab = (const float2*)p.tab;
  const float4* gmu = (const float4*)p.s.mu;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
  }
  if (warp == 0) tmem_alloc(&tslot, ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;

  // A generator: row 8 warp + (lane & 7) of this M tile (U at m = row, V at
  // m = 64 + row), particle pairs c = (lane >> 3) + 4 u
  const int arow = 8 * warp + (lane & 7);
  const int rg = mtile * 64 + arow;
  const bool rvalid = rg < p.tc_rows;
  const int2 rr = rvalid ? p.tc_row[rg] : make_int2(0, 0);
  const int ny = rr.x, nz = rr.y, ay = ny < 0 ? -ny : ny;
  const float nyf = (float)ny, nzf = (float)nz;
  const uint32_t idesc = tc_idesc_tf32(128, NS);
  const uint32_t sbo = kSfSK * 32;
  bool ok = true;   // this thread's waits all succeeded
  int ncom = 0;     // (thread 0) stages whose MMAs were issued

  // this thread's share of a stage's tables, loaded one stage ahead
  float2 tpre[kSfTabPer];
  float4 mpre = make_float4(0.f, 0.f, 0.f, 0.f);
  auto load_tables = [&](int s) {
    const int j0 = p0 + s * kSfSC;
#pragma unroll
    for (int u = 0; u < kSfTabPer; u++) {
      const int e = tid + u * kSfThreads;
      const int row = e / kSfSC, j = e - row * kSfSC;  // row = axis * K1 + |n|
      tpre[u] = (row < 3 * K1 && j0 + j < p1) ? gtab[(size_t)row * n + j0 + j] : make_float2(0.f, 0.f);
    }
    if (tid < kSfSC) mpre = j0 + tid < p1 ? gmu[j0 + tid] : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  if (nstage > 0) load_tables(0);

  for (int s = 0; s < nstage; s++) {
    unsigned char* st = smem + (s & 1) * sbytes;
    // the MMAs that last read this stage buffer (stage s - 2) are complete
    if (s >= 2 && ok) ok = mbar_wait(&bar[s & 1], ((s - 2) >> 1) & 1);
#pragma unroll
    for (int u = 0; u < kSfTabPer; u++) {
      const int e = tid + u * kSfThreads;
      const int row = e / kSfSC, j = e - row * kSfSC;
      if (row < 3 * K1) tabs[j * tstride + row] = tpre[u];
    }
    if (tid < kSfSC) mus[tid] = mpre;
    __syncthreads();
    if (s + 1 < nstage) load_tables(s + 1);  // in flight during this stage's generation
    unsigned char* ahi = st;
    unsigned char* alo = st + abytes;
    unsigned char* bhi = st + 2 * abytes;
    unsigned char* blo = st + 2 * abytes + bbytes;
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const int c = (lane >> 3) + 4 * u;  // particles 2c, 2c + 1 -> k = 4c .. 4c + 3
      float U[4] = {0.f, 0.f, 0.f, 0.f}, V[4] = {0.f, 0.f, 0.f, 0.f};
      if (rvalid) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const float2* tb = tabs + (2 * c + h) * tstride;
          float2 Y = tb[K1 + ay];
          if (ny < 0) Y.y = -Y.y;
          const float2 Z = tb[2 * K1 + nz];
          const float4 mu = mus[2 * c + h];
          const float pr = Y.x * Z.x - Y.y * Z.y, pi = Y.x * Z.y + Y.y * Z.x;
          const float cf = nyf * mu.y + nzf * mu.z;
          U[2 * h] = cf * pr;
          U[2 * h + 1] = cf * pi;
          V[2 * h] = mu.x * pr;
          V[2 * h + 1] = mu.x * pi;
        }
      }
      float4 h4, l4;
      tf32_split(U[0], h4.x, l4.x);
      tf32_split(U[1], h4.y, l4.y);
      tf32_split(U[2], h4.z, l4.z);
      tf32_split(U[3], h4.w, l4.w);
      *(float4*)(ahi + cm_off(arow, 4 * c, kSfSK)) = h4;
      *(float4*)(alo + cm_off(arow, 4 * c, kSfSK)) = l4;
      tf32_split(V[0], h4.x, l4.x);
      tf32_split(V[1], h4.y, l4.y);
      tf32_split(V[2], h4.z, l4.z);
      tf32_split(V[3], h4.w, l4.w);
      *(float4*)(ahi + cm_off(64 + arow, 4 * c, kSfSK)) = h4;
      *(float4*)(alo + cm_off(64 + arow, 4 * c, kSfSK)) = l4;
    }
    // B rows: 2q = (Re X, -Im X), 2q + 1 = (Im X, Re X) per particle, X = X(q - kc)
    for (int e = tid; e < NS * (kSfSK / 4); e += kSfThreads) {
      // a warp writes 8 rows x 4 particle pairs: whole 128-byte core-matrix rows
      const int nrow = (e & 7) + 8 * (e >> 6), c = ((e >> 3) & 3) + 4 * ((e >> 5) & 1);
      const int q = nrow >> 1, par = nrow & 1;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (q <= 2 * kc) {
        const int nx = q - kc, ax = nx < 0 ? -nx : nx;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const float2 X = tabs[(2 * c + h) * tstride + ax];
          const float xr = X.x, xi = nx < 0 ? -X.y : X.y;
          v[2 * h] = par ? xi : xr;
          v[2 * h + 1] = par ? xr : -xi;
        }
      }
      float4 h4, l4;
      tf32_split(v[0], h4.x, l4.x);
      tf32_split(v[1], h4.y, l4.y);
      tf32_split(v[2], h4.z, l4.z);
      tf32_split(v[3], h4.w, l4.w);
      *(float4*)(bhi + cm_off(nrow, 4 * c, kSfSK)) = h4;
      *(float4*)(blo + cm_off(nrow, 4 * c, kSfSK)) = l4;
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0 && ok) {
      tc_fence_after();
      const uint32_t ah = smem_u32(ahi), al = smem_u32(alo), bh = smem_u32(bhi), bl = smem_u32(blo);
#pragma unroll
      for (int ks = 0; ks < kSfSK / 8; ks++) {
        const uint32_t o = ks * 256;
        tc_mma_tf32(tmem, tc_desc(ah + o, 128, sbo), tc_desc(bh + o, 128, sbo), idesc, s > 0 || ks > 0);
        tc_mma_tf32(tmem, tc_desc(ah + o, 128, sbo), tc_desc(bl + o, 128, sbo), idesc, true);
        tc_mma_tf32(tmem, tc_desc(al + o, 128, sbo), tc_desc(bh + o, 128, sbo), idesc, true);
      }
      tc_commit(smem_u32(&bar[s & 1]));
      ncom = s + 1;
    }
  }
  // the last commit tracks every MMA of this block
  bool fin = ok && nstage > 0;
  if (fin) fin = mbar_wait(&bar[(nstage - 1) & 1], ((nstage - 1) >> 1) & 1);
  // after a failed wait: the MMAs that were issued finish before the exit
  if (tid == 0 && ncom > 0 && ncom < nstage) mbar_wait(&bar[(ncom - 1) & 1], ((ncom - 1) >> 1) & 1);
  ok = fin || nstage == 0;
  if (!ok && lane == 0) atomicOr(p.err, kErrTcWait);
  tc_fence_after();
  {
    // warp w: tensor-memory lanes 32 (w & 3) .., column half w >> 2
    const int m = 32 * (warp & 3) + lane;
    const int c0 = (warp >> 2) * (NS / 2);
    float* out = p.tc_part + (size_t)(chunk * p.tc_mt + mtile) * NS * 128;
    for (int cc = c0; cc < c0 + NS / 2; cc += 8) {
      float v[8];
      tmem_ld8(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + cc, v);
      tmem_wait_ld();
#pragma unroll
      for (int u = 0; u < 8; u++) out[(size_t)(cc + u) * 128 + m] = (fin) ? v[u] : 0.f;
    }
  }
  if (mtile == 0) {
    // FP64 moment sum of this chunk (surface term)
    double m0 = 0, m1 = 0, m2 = 0;
    for (int q = p0 + tid; q < p1; q += kSfThreads) {
      const float4 mu = gmu[q];
      m0 += (double)mu.x;
      m1 += (double)mu.y;
      m2 += (double)mu.z;
    }
    m0 = warp_sum(m0);
    m1 = warp_sum(m1);
    m2 = warp_sum(m2);
    if (lane == 0) {
      red[0][warp] = m0;
      red[1][warp] = m1;
      red[2][warp] = m2;
    }
    __syncthreads();
    if (tid < 3) {
      double s = 0;
      for (int w = 0; w < kSfThreads / 32; w++) s += red[tid][w];
      p.musum_part[3 * chunk + tid] = s;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tmem, ncols);
}

// One element of the scatter operand image: hi at [t][0], lo at [t][1].
__device__ __forceinline__ void w_put(float* img, int kp, int row, int k, float x) {
  float h, l;
  tf32_split(x, h, l);
  const int o = cm_off(row, k, kp) >> 2;
  img[o] = h;
  img[kScCols * kp + o] = l;
}

// Block per (M tile, column q): 64 rows x 4 groups of chunks, the groups
// combined in a fixed order.
template <bool FULL>
__global__ void __launch_bounds__(256) k_sf_tc_reduce(KParams p) {
  using L = ScatLayout<FULL>;
  __shared__ double red[4][4][64];
  const int Q = 2 * p.kc + 1;
  const int mtile = blockIdx.x / Q, q = blockIdx.x - mtile * Q;
  const int rl = threadIdx.x & 63, grp = threadIdx.x >> 6;
  if (blockIdx.x == 0 && threadIdx.x < 3) {
    double s = 0;
    for (int c = 0; c < p.tc_nchunk; c++) s += p.musum_part[3 * c + threadIdx.x];
    p.musum[threadIdx.x] = s;
  }
  const int NS = p.tc_ns;
  const size_t cstride = (size_t)p.tc_mt * NS * 128;
  const float* b = p.tc_part + (size_t)mtile * NS * 128;
  double ur = 0, ui = 0, vr = 0, vi = 0;
  for (int c = grp; c < p.tc_nchunk; c += 4) {
    const float* bc = b + (size_t)c * cstride;
    ur += (double)bc[(2 * q) * 128 + rl];
    ui += (double)bc[(2 * q + 1) * 128 + rl];
    vr += (double)bc[(2 * q) * 128 + 64 + rl];
    vi += (double)bc[(2 * q + 1) * 128 + 64 + rl];
  }
  red[grp][0][rl] = ur;
  red[grp][1][rl] = ui;
  red[grp][2][rl] = vr;
  red[grp][3][rl] = vi;
  __syncthreads();
  if (grp != 0) return;
  ur = ((red[0][0][rl] + red[1][0][rl]) + red[2][0][rl]) + red[3][0][rl];
  ui = ((red[0][1][rl] + red[1][1][rl]) + red[2][1][rl]) + red[3][1][rl];
  vr = ((red[0][2][rl] + red[1][2][rl]) + red[2][2][rl]) + red[3][2][rl];
  vi = ((red[0][3][rl] + red[1][3][rl]) + red[2][3][rl]) + red[3][3][rl];
  const int r = mtile * 64 + rl;
  if (r >= p.tc_rows) return;
  const int kk = p.tc_kmap[r * Q + q];
  if (kk < 0) return;
  const double nx = (double)(q - p.kc);
  const double sr = ur + nx * vr, si = ui + nx * vi;
  p.S[kk] = make_double2(sr, si);
  const double e = p.ek[kk];
  const double er = e * sr, ei = e * si;
  const int tt = r / L::RT, sl = r - tt * L::RT;
  const int kp = p.tc_kp;
  float* img = p.tc_w + (size_t)tt * 2 * kScCols * kp;
  double f = 1.0;
#pragma unroll
  for (int pp = 0; pp < L::P; pp++) {
    // W_p = nx^p conj(e S): (wr, wi)
    const float wr = (float)(f * er), wi = (float)(-f * ei);
    const int col = L::ccol(sl, pp);
    w_put(img, kp, 2 * col, 2 * q, wr);
    w_put(img, kp, 2 * col, 2 * q + 1, -wi);
    w_put(img, kp, 2 * col + 1, 2 * q, wi);
    w_put(img, kp, 2 * col + 1, 2 * q + 1, wr);
    f *= nx;
  }
}

// ---------------------------------------------------------------- scatter

// Warps 0-7: epilogue (warp w reads tensor-memory lanes 32 (w & 3) .. for
// its particles and the half w >> 2 of each tile); warp 8, one lane:
// producer (bulk copies of W tiles into NST stages, MMAs into two
// alternating accumulators).  An epilogue warp releases an accumulator as
// soon as it has loaded it, so the MMAs of the next tiles overlap the
// arithmetic of this one.
template <bool FULL>
__global__ void __launch_bounds__(kScThreads) k_kscat_tc(KParams p) {
  using L = ScatLayout<FULL>;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full_bar[kScMaxStages];  // W tile landed in a stage
  __shared__ __align__(8) uint64_t mma_bar[2];              // accumulator d complete
  __shared__ __align__(8) uint64_t free_bar[2];             // accumulator d loaded by all epilogue warps
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  __shared__ float part[6][kScParticles];                   // second tile halves' sums
  const int kp = p.tc_kp, kc = p.kc, K1 = kc + 1, n = p.n, R = p.tc_rows, NT = p.tc_nt, NST = p.tc_nst;
  const int abytes = kScParticles * kp * 4;
  const int tbytes = 2 * kScCols * kp * 4;
  unsigned char* a_hi = smem;
  unsigned char* a_lo = smem + abytes;
  unsigned char* stage0 = smem + 2 * abytes;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool producer = warp == kScEpiWarps;
  const int quarter = warp & 3, half = (warp >> 2) & 1;
  const int pl = 32 * quarter + lane;  // particle of this epilogue thread = tensor-memory lane
  const int i = blockIdx.x * kScParticles + pl;
  const bool act = !producer && i < n;
  const int ii = i < n ? i : n - 1;
  const float2* gtab = (const float2*)p.tab;

  if (tid == 0) {
    for (int q = 0; q < kScMaxStages; q++) mbar_init(&full_bar[q], 1);
    for (int q = 0; q < 2; q++) {
      mbar_init(&mma_bar[q], 1);
      mbar_init(&free_bar[q], kScEpiWarps);
    }
    mbar_init_fence();
    abort_flag = 0;
  }
  if (warp == 0) tmem_alloc(&tslot, 2 * kScCols);
  if (!producer) {
    // A row of this particle: X(nx), nx = q - kc, at k = 2q (Re), 2q + 1 (Im);
    // the two warps of a particle write half of the row each
    for (int c = half * (kp / 8); c < (half + 1) * (kp / 8); c++) {
      float v[4];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int q = 2 * c + h;
        float xr = 0.f, xi = 0.f;
        if (i < n && q <= 2 * kc) {
          const int nx = q - kc;
          const float2 X = gtab[(size_t)(nx < 0 ? -nx : nx) * n + i];
          xr = X.x;
          xi = nx < 0 ? -X.y : X.y;
        }
        v[2 * h] = xr;
        v[2 * h + 1] = xi;
      }
      float4 h4, l4;
      tf32_split(v[0], h4.x, l4.x);
      tf32_split(v[1], h4.y, l4.y);
      tf32_split(v[2], h4.z, l4.z);
      tf32_split(v[3], h4.w, l4.w);
      *(float4*)(a_hi + cm_off(pl, 4 * c, kp)) = h4;
      *(float4*)(a_lo + cm_off(pl, 4 * c, kp)) = l4;
    }
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;
  float b[3] = {0.f, 0.f, 0.f}, cb[3] = {0.f, 0.f, 0.f}, f[3] = {0.f, 0.f, 0.f}, cfr[3] = {0.f, 0.f, 0.f};

  if (producer) {
    if (lane == 0) {
      const uint32_t idesc = tc_idesc_tf32(128, kScCols);
      const uint32_t sbo = kp * 32;
      const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo);
      bool ok = true;
      int issued = 0, consumed = 0, ncom = 0;
      for (int u = 0; u < NST && u < NT; u++) {
        mbar_expect_tx(&full_bar[u], tbytes);
        bulk_g2s(stage0 + u * tbytes, p.tc_w + (size_t)u * (tbytes / 4), tbytes, &full_bar[u]);
        issued = u + 1;
      }
      for (int t = 0; t < NT && ok; t++) {
        ok = mbar_wait_abort(&full_bar[t % NST], (t / NST) & 1, &abort_flag);
        if (!ok) break;
        consumed = t + 1;
        // accumulator t & 1 was loaded by the epilogue of tile t - 2
        if (t >= 2) ok = mbar_wait_abort(&free_bar[t & 1], ((t - 2) >> 1) & 1, &abort_flag);
        if (!ok) break;
        tc_fence_after();
        const uint32_t bh = smem_u32(stage0 + (t % NST) * tbytes), bl = bh + kScCols * kp * 4;
        const uint32_t d = tmem + (uint32_t)((t & 1) * kScCols);
        for (int ks = 0; ks < kp / 8; ks++) {
          const uint32_t o = ks * 256;
          tc_mma_tf32(d, tc_desc(ah + o, 128, sbo), tc_desc(bh + o, 128, sbo), idesc, ks > 0);
          tc_mma_tf32(d, tc_desc(ah + o, 128, sbo), tc_desc(bl + o, 128, sbo), idesc, true);
          tc_mma_tf32(d, tc_desc(al + o, 128, sbo), tc_desc(bh + o, 128, sbo), idesc, true);
        }
        tc_commit(smem_u32(&mma_bar[t & 1]));
        ncom = t + 1;
        // the stage of tile t - 1 is free once its MMAs are done: next tile in
        const int u = t - 1 + NST;
        if (t >= 1 && u < NT) {
          ok = mbar_wait_abort(&mma_bar[(t - 1) & 1], ((t - 1) >> 1) & 1, &abort_flag);
          if (!ok) break;
          mbar_expect_tx(&full_bar[u % NST], tbytes);
          bulk_g2s(stage0 + (u % NST) * tbytes, p.tc_w + (size_t)u * (tbytes / 4), tbytes, &full_bar[u % NST]);
          issued = u + 1;
        }
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(p.err, kErrTcWait);
      }
      // nothing of this block may still be in flight when it exits
      for (int u = consumed; u < issued; u++) mbar_wait(&full_bar[u % NST], (u / NST) & 1);
      if (ncom > 0) mbar_wait(&mma_bar[(ncom - 1) & 1], ((ncom - 1) >> 1) & 1);
    }
  } else {
    const float4 mu = act ? ((const float4*)p.s.mu)[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    auto kahan = [](float& s, float& c, float v) {
      const float y = v - c, t = s + y;
      c = (t - s) - y;
      s = t;
    };
    for (int t = 0; t < NT; t++) {
      bool w = mbar_wait_abort(&mma_bar[t & 1], (t >> 1) & 1, &abort_flag);
      w = __all_sync(kFull, w);
      if (!w) {
        if (lane == 0) {
          abort_flag = 1;
          atomicOr(p.err, kErrTcWait);
        }
        break;
      }
      tc_fence_after();
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)((t & 1) * kScCols + 32 * half), v);
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&free_bar[t & 1]);
      float tb0 = 0.f, tb1 = 0.f, tb2 = 0.f, tf0 = 0.f, tf1 = 0.f, tf2 = 0.f;
      int cur_nz = -1;
      float2 Z = make_float2(0.f, 0.f);
#pragma unroll
      for (int sh = 0; sh < L::RH; sh++) {
        const int r = t * L::RT + half * L::RH + sh;
        if (r < R) {
          const int2 rr = p.tc_row[r];
          const int ny = rr.x, nz = rr.y;
          float2 Y = gtab[(size_t)(K1 + (ny < 0 ? -ny : ny)) * n + ii];
          if (ny < 0) Y.y = -Y.y;
          if (nz != cur_nz) {
            Z = gtab[(size_t)(2 * K1 + nz) * n + ii];
            cur_nz = nz;
          }
          const float pr = Y.x * Z.x - Y.y * Z.y, pi = Y.x * Z.y + Y.y * Z.x;
          const float nyf = (float)ny, nzf = (float)nz;
          const float* qv = v + 2 * L::P * sh;
          const float re0 = pr * qv[0] - pi * qv[1];
          const float re1 = pr * qv[2] - pi * qv[3];
          tb0 += re1;
          tb1 += nyf * re0;
          tb2 += nzf * re0;
          if constexpr (FULL) {
            const float im0 = pr * qv[1] + pi * qv[0], im1 = pr * qv[3] + pi * qv[2];
            const float im2 = pr * qv[5] + pi * qv[4];
            const float cf = nyf * mu.y + nzf * mu.z;
            tf0 += mu.x * im2 + cf * im1;
            const float g = mu.x * im1 + cf * im0;
            tf1 += nyf * g;
            tf2 += nzf * g;
          }
        }
      }
      kahan(b[0], cb[0], tb0);
      kahan(b[1], cb[1], tb1);
      kahan(b[2], cb[2], tb2);
      if constexpr (FULL) {
        kahan(f[0], cfr[0], tf0);
        kahan(f[1], cfr[1], tf1);
        kahan(f[2], cfr[2], tf2);
      }
    }
    if (half == 1) {
#pragma unroll
      for (int a = 0; a < 3; a++) {
        part[a][pl] = b[a] - cb[a];
        part[3 + a][pl] = f[a] - cfr[a];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (act && half == 0) {
    // the two halves of the tiles, added in a fixed order
    float* B = (float*)p.B;
    const float cfl = (float)p.cflux;
    B[i] = -cfl * ((b[0] - cb[0]) + part[0][pl]);
    B[n + i] = -cfl * ((b[1] - cb[1]) + part[1][pl]);
    B[2 * n + i] = -cfl * ((b[2] - cb[2]) + part[2][pl]);
    if constexpr (FULL) {
      float* F = (float*)p.F;
      const float cfo = (float)p.cforce;
      F[i] = cfo * ((f[0] - cfr[0]) + part[3][pl]);
      F[n + i] = cfo * ((f[1] - cfr[1]) + part[4][pl]);
      F[2 * n + i] = cfo * ((f[2] - cfr[2]) + part[5][pl]);
    }
  }
  if (warp == 0) tmem_free(tmem, 2 * kScCols);
}

// ------------------------------------------------------------ host side

bool kspace_tc_supported(int kc) {
  return kc >= 1 && kc <= kTcMaxKc && sf_smem(kc) <= kSmemLimit && scat_smem(kc, 2) <= kSmemLimit && tc_ns(kc) <= 256;
}

TcShape kspace_tc_shape(int kc, int n, int rows, int nsm) {
  TcShape s{};
  s.ns = tc_ns(kc);
  s.kp = tc_kp(kc);
  s.mt = (rows + 63) / 64;
  s.nst = scat_smem(kc, 3) <= kSmemLimit ? 3 : 2;
  s.nt_full = (rows + ScatLayout<true>::RT - 1) / ScatLayout<true>::RT;
  s.nt_field = (rows + ScatLayout<false>::RT - 1) / ScatLayout<false>::RT;
  s.rt_full = ScatLayout<true>::RT;
  s.rt_field = ScatLayout<false>::RT;
  // structure-factor grid: M tiles x chunks of <= 1024 particles, the chunk
  // count filling whole waves of resident blocks
  int res = (int)((228 * 1024) / (sf_smem(kc) + 1024 + 2048));
  res = std::max(1, std::min(res, 2));
  const long slots = (long)nsm * res;
  const long nch_min = std::max(1L, ((long)n + 1023) / 1024);
  const long waves = std::max(1L, ((long)s.mt * nch_min + slots - 1) / slots);
  long nch = std::max(nch_min, waves * slots / (long)std::max(1, s.mt));
  nch = std::min<long>(nch, std::max(1L, ((long)n + kSfSC - 1) / kSfSC));
  s.chunk = (int)((((long)n + nch - 1) / nch + kSfSC - 1) / kSfSC * kSfSC);
  s.nchunk = (n + s.chunk - 1) / s.chunk;
  return s;
}

size_t kspace_tc_image_floats(int kc, int nt) { return (size_t)nt * 2 * kScCols * tc_kp(kc); }

int launch_kspace_tc(cudaStream_t st, const KParams& p, bool full, cudaEvent_t* ev) {
  const size_t sm1 = sf_smem(p.kc);
  cudaFuncSetAttribute(k_sf_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  k_sf_tc<<<dim3(p.tc_mt, p.tc_nchunk), kSfThreads, sm1, st>>>(p);
  if (ev) cudaEventRecordWithFlags(ev[0], st, cudaEventRecordExternal);
  const int nred = p.tc_mt * (2 * p.kc + 1);
  if (full)
    k_sf_tc_reduce<true><<<nred, 256, 0, st>>>(p);
  else
    k_sf_tc_reduce<false><<<nred, 256, 0, st>>>(p);
  if (ev) cudaEventRecordWithFlags(ev[1], st, cudaEventRecordExternal);
  const size_t sm2 = scat_smem(p.kc, p.tc_nst);
  const int nb = (p.n + kScParticles - 1) / kScParticles;
  if (full) {
    cudaFuncSetAttribute(k_kscat_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
    k_kscat_tc<true><<<nb, kScThreads, sm2, st>>>(p);
  } else {
    cudaFuncSetAttribute(k_kscat_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
    k_kscat_tc<false><<<nb, kScThreads, sm2, st>>>(p);
  }
  return 3;
}

}  // namespace md
