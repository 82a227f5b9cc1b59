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
// Precision: each FP32 operand is split into a hi + lo pair (FP16 pairs in
// the structure factor, kind::f16; TF32 pairs in the scatter, kind::tf32,
// whose W operand spans more decades than FP16 holds) and the products are
// hi*hi + hi*lo + lo*hi (three MMAs into one FP32 accumulator), ~21-22
// significant bits per product like FP32 arithmetic.  The tensor core's FP32
// accumulation loses precision with the number of MMAs added into one
// accumulator (measured at N = 32768: 5.5e-6 relative error of S with 392
// particles per accumulator, 1.8e-6 with 128), so the structure factor uses
// chunks of <= 512 particles (4 accumulators of <= 128 each, added in FP32)
// and sums the chunks exactly (error-free FP32 pairs, then FP64), like the
// reference's FP64 sums over particles; the scatter sums over the nx of a
// row in the MMA (<= 2 kc + 1 terms), over the rows of a tile in FP32 and
// over tiles with compensated FP32 sums.  All sums have a fixed order:
// results are deterministic.
//
// Kernels:
//   k_tc_prep    once per step (positions are frozen across the step's
//                evaluations): the X operand tiles (hi, lo) of every stage
//                of 32 particles in the shared-memory layout of the
//                structure factor, and their Y, Z phases in blocks.
//   k_sf_tc      grid (M tiles, chunks); 16 warps generate the U, V operand
//                of 32 particles per stage into a ring of shared-memory
//                slots, one warp bulk-copies each stage's X tiles, tables and
//                moments into a second ring, 4 warps issue the MMAs (stages
//                dealt round-robin, one accumulator each, added in a fixed
//                order at the end); mbarriers hand stages between the roles
//                and tcgen05.commit releases the slots.
//   k_sf_tc_reduce  exact sum of the chunk partials (TwoSum pairs, then
//                FP64), S(n) = C_U + nx C_V and e(n) S(n) in FP64, and the scatter's W operand image (hi, lo) in
//                the shared-memory layout the scatter copies in bulk.
//   k_kscat_tc   128 particles per block, their X phases (the A operand, hi
//                and lo) in tensor memory; W tiles of 128 columns stream in
//                by bulk copy (2-3 stages); two issuing warps alternate tiles
//                into two tensor-memory accumulators, and 16 epilogue warps
//                (4 per tile quarter) turn each accumulator into per-row terms
//                of B and F.
//
// What sets the pace (GB300, measured at N = 32768, kc = 16): an mbarrier
// hand-off between warps takes ~0.1 us, an MMA commit round trip ~0.2 us
// plus the MMAs (one 32-particle stage of the structure factor: 12 MMAs,
// ~0.3 us alone), a bulk copy of a stage from L2 ~0.3 us.  A structure-factor
// block (16 stages) takes ~19 us: ~0.9 us per stage, in which every role
// (generators, issuers, copies) runs well below its own rate and no single
// wait dominates (a per-block timeline of each role's stage events), plus
// ~5 us of setup, pipeline fill, drain and tensor-memory read-out.  The
// scatter's CUDA-core epilogue is the bound of the scatter.
#include "md_common.cuh"
#include "md_kernels.h"
#include "md_tc.cuh"

#include <algorithm>
#include <type_traits>
#include <cstring>

namespace md {

constexpr int kSfSC = 32;            // particles per structure-factor stage (a multiple of 16)
constexpr int kSfSK = 2 * kSfSC;     // K elements per stage
constexpr int kSfGenWarps = 16;      // structure factor: operand generators (64 rows x U, V)
constexpr int kSfIssuers = 4;        // structure factor: MMA-issuing warps (one accumulator each)
constexpr int kSfThreads = 32 * (kSfGenWarps + 1 + kSfIssuers);  // + copy producer + issuers
constexpr int kSfMaxSlots = 8;       // deepest operand rings
constexpr int kSfMaxChunk = 512;     // particles per structure-factor chunk (4 accumulators of <= 128)
constexpr int kTabPad = kSfSC + 2;   // Y, Z block row stride: even (16-byte pairs), 4 banks apart
constexpr int kSfPairs = kSfSC / 2;  // particle pairs per stage (4 K elements each)
static_assert(kSfSC % 16 == 0, "stages of whole 16-particle generator passes");
constexpr int kTcMaxKc = 25;         // operand bounds: A of the scatter in 256 tensor-memory columns
constexpr int kScEpiWarps = 16;      // scatter: 4 warps per tensor-memory lane quarter (tile quarters)
constexpr int kScThreads = 32 * (kScEpiWarps + 3);  // + copy producer + two MMA issuers
constexpr int kScParticles = 128;    // particles per scatter block (tensor-memory lanes)
constexpr int kScCols = 128;         // scatter tile: 128 output columns (MMA N)
constexpr int kScMaxStages = 4;
constexpr size_t kSmemLimit = 227 * 1024 - 5 * 1024;  // dynamic shared memory per block (static <= 4 KB)

// Scatter tile: 128 real columns in four quarters of 16 complex columns; a
// quarter holds RQ k rows x P complex columns Q_0 .. Q_{P-1} (+ padding),
// one 32-column tensor-memory load of an epilogue warp.
template <bool FULL>
struct ScatLayout {
  static constexpr int P = FULL ? 3 : 2;       // Q_p per row
  static constexpr int RQ = FULL ? 5 : 8;      // rows per quarter tile
  static constexpr int RT = 4 * RQ;            // rows per tile
  // complex column of Q_p of the tile's row sl
  __host__ __device__ static constexpr int ccol(int sl, int pp) { return (sl / RQ) * 16 + (sl % RQ) * P + pp; }
};

// Row descriptors of the scatter (built once by the host, read with
// warp-uniform loads): both tile shapes' rows, padded to whole tiles
// (padding rows have zero W columns).
__host__ __device__ inline int scat_rows_pad(int R) {
  const int a = (R + ScatLayout<true>::RT - 1) / ScatLayout<true>::RT * ScatLayout<true>::RT;
  const int b = (R + ScatLayout<false>::RT - 1) / ScatLayout<false>::RT * ScatLayout<false>::RT;
  return a > b ? a : b;
}

static int tc_ns(int kc) { return (2 * (2 * kc + 1) + 15) / 16 * 16; }
static int tc_kp(int kc) { return (2 * (2 * kc + 1) + 7) / 8 * 8; }

// Structure-factor shared memory: a ring of na generated U, V operand slots
// (hi, lo) and a ring of nb copied-in slots (X tiles hi, lo | Y, Z block |
// moments), so the bulk copies run nb - 1 stages ahead and the generators
// na - 1 stages ahead of the MMAs.
struct SfLayout {
  int na, nb, a, b, t, m, bt, bytes;
  __host__ __device__ SfLayout(int ns, int k1, int na_, int nb_)
      : na(na_), nb(nb_), a(128 * kSfSK * 2), b(ns * kSfSK * 2), t(2 * k1 * kTabPad * 8), m(kSfSC * 16),
        bt(2 * b + t + m), bytes(na_ * 2 * a + nb_ * bt) {}
  // byte offsets of generated slot q and copied slot q (the roles keep the
  // slot index and phase of their stage as counters: the ring depths are
  // runtime values, and a division per stage costs the generators as much
  // as their arithmetic)
  __host__ __device__ int aslot_at(int q) const { return q * 2 * a; }
  __host__ __device__ int btslot_at(int q) const { return na * 2 * a + q * bt; }
};
// Deepest rings that fit.  The generated ring's depth is a multiple of the
// issuer count: an issuer waits on full_a of its stage s by parity, which is
// only unambiguous if the slot's previous phase (stage s - na) is already
// complete, i.e. was this issuer's own earlier stage.  (With na = 3 and four
// issuers, an issuer could pass the wait one phase early and read a slot
// that still held stage s - na.)  The copied ring is waited on only by the
// copy producer and the generators, which take every stage in order.
// ring >= 0 picks option `ring` of the list when it fits (a tuning choice);
// otherwise the deepest option that fits.
constexpr int kSfRingOpts = 6;
static SfLayout sf_layout(int kc, int ring = -1) {
  const int ns = tc_ns(kc), k1 = kc + 1;
  const int opts[kSfRingOpts][2] = {{8, 6}, {8, 5}, {8, 4}, {4, 4}, {4, 3}, {4, 2}};
  static_assert(8 % kSfIssuers == 0 && 4 % kSfIssuers == 0, "generated ring depths: multiples of the issuers");
  if (ring >= 0 && ring < kSfRingOpts) {
    SfLayout l(ns, k1, opts[ring][0], opts[ring][1]);
    if ((size_t)l.bytes <= kSmemLimit) return l;
  }
  for (const auto& o : opts) {
    SfLayout l(ns, k1, o[0], o[1]);
    if ((size_t)l.bytes <= kSmemLimit) return l;
  }
  return SfLayout(ns, k1, 4, 1);
}
static size_t sf_smem(int kc) { return (size_t)sf_layout(kc).bytes; }

// Ring options of the structure factor that fit for kc (tuning candidates).
int kspace_tc_ring_options(int kc, int* opts_out, int cap) {
  const int ns = tc_ns(kc), k1 = kc + 1;
  const int opts[kSfRingOpts][2] = {{8, 6}, {8, 5}, {8, 4}, {4, 4}, {4, 3}, {4, 2}};
  int m = 0;
  for (int q = 0; q < kSfRingOpts; q++)
    if ((size_t)SfLayout(ns, k1, opts[q][0], opts[q][1]).bytes <= kSmemLimit && m < cap) opts_out[m++] = q;
  return m;
}
// Scatter shared memory: nst W-tile stages | (yz) the Y, Z phases of the
// block's particles [2 (kc + 1)][128] float2.
static size_t scat_smem(int kc, int nst, int /*rows*/, bool yz = false) {
  const int kp = tc_kp(kc);
  return (size_t)nst * 2 * kScCols * kp * 4 +
         (yz ? (size_t)2 * (kc + 1) * kScParticles * 8 : 0);
}

// ------------------------------------------------------ per-step operands

// Block per stage of kSfSC particles: X operand rows 2q = (Re X, -Im X),
// 2q + 1 = (Im X, Re X) per particle (q = nx + kc; zero beyond 2 kc and
// beyond n) as FP16 hi, lo tiles [ns][2 kSfSC]; Y(|ny|), Z(nz) of the stage's
// particles.
__device__ __forceinline__ void tc_prep_body(const KParams& p, int sb) {
  const int NS = p.tc_ns, kc = p.kc, K1 = kc + 1, n = p.n;
  const int j0 = sb * kSfSC;
  const float2* gtab = (const float2*)p.tab;
  // FP16 tiles [hi, lo][NS][32]: 2 bytes per element
  unsigned char* bimg = (unsigned char*)p.tc_bimg + (size_t)sb * 2 * NS * kSfSK * 2;
  for (int e = threadIdx.x; e < NS * (kSfSK / 4); e += blockDim.x) {
    // 8 rows x kSfPairs particle pairs per 8-row group: whole core-matrix rows
    const int nrow = (e & 7) + 8 * (e / (8 * kSfPairs)), c = (e >> 3) % kSfPairs;
    const int q = nrow >> 1, par = nrow & 1;
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (q <= 2 * kc) {
      const int nx = q - kc, ax = nx < 0 ? -nx : nx;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int j = j0 + 2 * c + h;
        if (j < n) {
          const float2 X = gtab[(size_t)ax * n + j];
          const float xr = X.x, xi = nx < 0 ? -X.y : X.y;
          v[2 * h] = par ? xi : xr;
          v[2 * h + 1] = par ? xr : -xi;
        }
      }
    }
    uint2 hi, lo;
    f16_split2(v[0], v[1], hi.x, lo.x);
    f16_split2(v[2], v[3], hi.y, lo.y);
    *(uint2*)(bimg + cm_off16(nrow, 4 * c, kSfSK)) = hi;
    *(uint2*)(bimg + NS * kSfSK * 2 + cm_off16(nrow, 4 * c, kSfSK)) = lo;
  }
  float2* tb = p.tc_tblk + (size_t)sb * 2 * K1 * kTabPad;
  for (int e = threadIdx.x; e < 2 * K1 * kTabPad; e += blockDim.x) {
    const int row = e / kTabPad, jj = e - row * kTabPad;  // row = axis (Y, Z) * K1 + |n|
    const int j = j0 + jj;
    tb[e] = (jj < kSfSC && j < n) ? gtab[(size_t)(K1 + row) * n + j] : make_float2(0.f, 0.f);
  }
}

__global__ void __launch_bounds__(256) k_tc_prep(KParams p) { tc_prep_body(p, blockIdx.x); }
// Packed systems: one block per task (system, stage block).
__global__ void __launch_bounds__(256) k_tc_prep_packed(const KParams* __restrict__ ps, const Task* __restrict__ tk) {
  const Task t = tk[blockIdx.x];
  tc_prep_body(ps[t.rep], t.blk);
}

// ------------------------------------------------------ structure factor

// Roles (warps): 0-15 generate the U, V operand of a stage into a
// generated-operand slot; 16 bulk-copies X tiles, Y, Z blocks and moments
// into copied-operand slots; 17 .. 16 + kSfIssuers issue the MMAs, issuer i
// taking the stages s = i (mod kSfIssuers) into its own accumulator (several
// issuing threads keep the tensor cores busy with these N <= 112 MMAs); the
// accumulators are added in a fixed order at the end.
__device__ __forceinline__ void sf_tc_body(const KParams& p, int mtile, int chunk) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full_bt[kSfMaxSlots];   // X tiles, tables, moments landed
  __shared__ __align__(8) uint64_t bt_empty[kSfMaxSlots];  // MMAs that read the copied slot are complete
  __shared__ __align__(8) uint64_t full_a[kSfMaxSlots];    // U, V operand written (all generator warps)
  __shared__ __align__(8) uint64_t a_empty[kSfMaxSlots];   // MMAs that read the generated slot are complete
  __shared__ __align__(8) uint64_t dfull[kSfIssuers];      // all MMAs of issuer i complete
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  __shared__ double red[3][kSfGenWarps];
  const int NS = p.tc_ns, kc = p.kc, K1 = kc + 1, n = p.n;
  const SfLayout L(NS, K1, p.tc_sfa, p.tc_sfb);
  const int kSfA = L.na, kSfB = L.nb;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p0 = chunk * p.tc_chunk, p1 = min(n, p0 + p.tc_chunk);
  const int nstage = p1 > p0 ? (p1 - p0 + kSfSC - 1) / kSfSC : 0;
  const uint32_t acols = NS <= 64 ? 64 : 128;  // columns per accumulator
  const uint32_t ncols = kSfIssuers * acols <= 256 ? 256 : 512;

  if (tid == 0) {
    for (int q = 0; q < kSfB; q++) {
      mbar_init(&full_bt[q], 1);
      mbar_init(&bt_empty[q], 1);
    }
    for (int q = 0; q < kSfA; q++) {
      mbar_init(&full_a[q], kSfGenWarps);
      mbar_init(&a_empty[q], 1);
    }
    for (int q = 0; q < kSfIssuers; q++) mbar_init(&dfull[q], 1);
    mbar_init_fence();
    abort_flag = 0;
  }
  if (warp == 0) tmem_alloc(&tslot, ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;

  if (warp == kSfGenWarps) {
    // copy producer
    if (lane == 0) {
      auto issue_copy = [&](int s, int q) {  // stage s into copied slot q
        unsigned char* st = smem + L.btslot_at(q);
        uint64_t* bar = &full_bt[q];
        const int j0 = p0 + s * kSfSC, sb = j0 / kSfSC;
        const uint32_t mb = (uint32_t)(min(kSfSC, p1 - j0) * 16);
        mbar_expect_tx(bar, (uint32_t)(2 * L.b + L.t) + mb);
        bulk_g2s(st, (const unsigned char*)p.tc_bimg + (size_t)sb * 2 * NS * kSfSK * 2, 2 * L.b, bar);
        bulk_g2s(st + 2 * L.b, p.tc_tblk + (size_t)sb * 2 * K1 * kTabPad, L.t, bar);
        bulk_g2s(st + 2 * L.b + L.t, (const float4*)p.s.mu + j0, mb, bar);
      };
      bool ok = true;
      int issued = 0;
      for (int s = 0; s < kSfB && s < nstage; s++) {
        issue_copy(s, s);
        issued = s + 1;
      }
      int q = 0, ph = 0;  // slot and phase parity of stage s
      for (int s = 0; s + kSfB < nstage && ok; s++) {
        // the copied slot of stage s takes stage s + kSfB once stage s's MMAs are done
        ok = mbar_wait_abort(&bt_empty[q], ph, &abort_flag, p.tc_wait);
        if (!ok) break;
        issue_copy(s + kSfB, q);
        issued = s + kSfB + 1;
        if (++q == kSfB) {
          q = 0;
          ph ^= 1;
        }
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(p.err, kErrTcWait);
      }
      // no copy may still be in flight at the exit: the last copy of each slot has landed
      for (int u = issued - kSfB > 0 ? issued - kSfB : 0; u < issued; u++)
        mbar_wait(&full_bt[u % kSfB], (u / kSfB) & 1, p.tc_wait);
    }
  } else if (warp > kSfGenWarps) {
    // MMA issuer is: stages is, is + kSfIssuers, ...
    const int is = warp - kSfGenWarps - 1;
    if (lane == 0) {
      const uint32_t idesc = tc_idesc_f16(128, NS);
      const uint32_t sbo = kSfSK * 16;  // 8-row groups of kSfSK 2-byte elements
      const uint32_t d = tmem + (uint32_t)is * acols;
      bool ok = true, any = false;
      // generated slot qa (kSfA is a multiple of kSfIssuers: exact wraps) and
      // its phase parity, copied slot qb of stage s
      int qa = is, pha = 0, qb = is % kSfB;
      for (int s = is; s < nstage && ok; s += kSfIssuers) {
        ok = mbar_wait_abort(&full_a[qa], pha, &abort_flag, p.tc_wait);
        if (!ok) break;
        tc_fence_after();
        // descriptors of the slots' tiles; k step ks (16 elements) starts 256 B (16 address units) further
        const uint64_t dah = tc_desc(smem_u32(smem + L.aslot_at(qa)), 128, sbo), dal = dah + (uint64_t)(L.a >> 4);
        const uint64_t dbh = tc_desc(smem_u32(smem + L.btslot_at(qb)), 128, sbo), dbl = dbh + (uint64_t)(L.b >> 4);
#pragma unroll
        for (int ks = 0; ks < kSfSK / 16; ks++) {
          const uint64_t o = 16 * ks;
          tc_mma_f16(d, dah + o, dbh + o, idesc, any || ks > 0);
          tc_mma_f16(d, dah + o, dbl + o, idesc, true);
          tc_mma_f16(d, dal + o, dbh + o, idesc, true);
        }
        any = true;
        tc_commit(smem_u32(&bt_empty[qb]));
        tc_commit(smem_u32(&a_empty[qa]));
        qa += kSfIssuers;
        if (qa >= kSfA) {
          qa -= kSfA;
          pha ^= 1;
        }
        qb += kSfIssuers;
        while (qb >= kSfB) qb -= kSfB;
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(p.err, kErrTcWait);
      }
      tc_commit(smem_u32(&dfull[is]));  // tracks every MMA this issuer started
    }
  } else {
    // generator: row 8 (warp & 7) + (lane & 7) of this M tile (U at m = row,
    // V at m = 64 + row), particle pairs c = (lane >> 3) + 4 (warp >> 3) + 8 u
    const int arow = 8 * (warp & 7) + (lane & 7);
    const int c0 = (lane >> 3) + 4 * (warp >> 3);  // pair c: particles 2c, 2c + 1 -> k = 4c .. 4c + 3
    const int rg = mtile * 64 + arow;
    // rows beyond R (last M tile) take row (0, 0): finite operands whose
    // accumulator rows the reduction never reads (a row of A reaches only its
    // own row of the product)
    const int2 rr = rg < p.tc_rows ? p.tc_row[rg] : make_int2(0, 0);
    const int ny = rr.x, nz = rr.y, ay = ny < 0 ? -ny : ny;
    const float nyf = (float)ny, nzf = (float)nz;
    const float ysg = ny < 0 ? -1.f : 1.f;  // conj Y for ny < 0
    // this thread's first particle in the stage's Y, Z rows and moments
    const int yo = ay * kTabPad + 2 * c0, zo = (K1 + nz) * kTabPad + 2 * c0, mo = 2 * c0;
    // store offset of pair c0 in the U rows; pair c0 + 8 u is kPairStep u
    // bytes further (4 core matrices along K), the V rows kVRows further
    constexpr int kPairStep = 8 * 4 / 8 * 128, kVRows = 64 / 8 * kSfSK * 16;
    static_assert(kSfPairs % 8 == 0, "whole passes of 8 pairs");
    const int so = cm_off16(arow, 4 * c0, kSfSK);
    // U, V of this thread's pairs; CHECKED zeroes particles j >= jlim (the
    // last stage of a chunk: its slot beyond jlim holds older data)
    auto gen = [&](auto checked, unsigned char* sa, const float2* tb, const float4* mus, int jlim) {
      constexpr bool CHECKED = decltype(checked)::value;
      constexpr int NP = kSfPairs / 8;  // passes of two particles
      // every load of the stage first: the operand stores below go to the
      // same shared memory, so loads after a store could not be moved up
      float2 Ys[2 * NP], Zs[2 * NP];
      float4 Ms[2 * NP];
#pragma unroll
      for (int u = 0; u < NP; u++) {
        // the pass's two particles are adjacent: one 16-byte load per table
        // row (the rows of a generator warp's 8 lanes fall 4 banks apart)
        const float4 y2 = *(const float4*)(tb + yo + 16 * u), z2 = *(const float4*)(tb + zo + 16 * u);
        Ys[2 * u] = make_float2(y2.x, y2.y);
        Ys[2 * u + 1] = make_float2(y2.z, y2.w);
        Zs[2 * u] = make_float2(z2.x, z2.y);
        Zs[2 * u + 1] = make_float2(z2.z, z2.w);
        Ms[2 * u] = mus[mo + 16 * u];
        Ms[2 * u + 1] = mus[mo + 16 * u + 1];
      }
#pragma unroll
      for (int u = 0; u < NP; u++) {
        float U[4], V[4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int jj = 16 * u + h;
          const float2 Y = Ys[2 * u + h];
          const float2 Z = Zs[2 * u + h];
          float4 mu = Ms[2 * u + h];
          const float yi = ysg * Y.y;
          float pr = fmaf(Y.x, Z.x, -yi * Z.y), pi = fmaf(Y.x, Z.y, yi * Z.x);
          if constexpr (CHECKED) {
            const bool in = mo + jj < jlim;
            pr = in ? pr : 0.f;
            pi = in ? pi : 0.f;
            mu = in ? mu : make_float4(0.f, 0.f, 0.f, 0.f);
          }
          const float cf = fmaf(nyf, mu.y, nzf * mu.z);
          U[2 * h] = cf * pr;
          U[2 * h + 1] = cf * pi;
          V[2 * h] = mu.x * pr;
          V[2 * h + 1] = mu.x * pi;
        }
        uint2 hi, lo;
        unsigned char* d = sa + so + kPairStep * u;
        f16_split2(U[0], U[1], hi.x, lo.x);
        f16_split2(U[2], U[3], hi.y, lo.y);
        *(uint2*)d = hi;
        *(uint2*)(d + L.a) = lo;
        f16_split2(V[0], V[1], hi.x, lo.x);
        f16_split2(V[2], V[3], hi.y, lo.y);
        *(uint2*)(d + kVRows) = hi;
        *(uint2*)(d + kVRows + L.a) = lo;
      }
    };
    // slots and phase parities of stage s; the a_empty phase that frees the
    // generated slot for stage s is the one of stage s - kSfA (parity pha ^ 1)
    int qa = 0, pha = 0, qb = 0, phb = 0;
    for (int s = 0; s < nstage; s++) {
      bool w = mbar_wait_abort(&full_bt[qb], phb, &abort_flag, p.tc_wait);
      if (w && s >= kSfA) w = mbar_wait_abort(&a_empty[qa], pha ^ 1, &abort_flag, p.tc_wait);
      w = __all_sync(kFull, w);
      if (!w) {
        if (lane == 0) {
          abort_flag = 1;
          atomicOr(p.err, kErrTcWait);
        }
        break;
      }
      unsigned char* sa = smem + L.aslot_at(qa);
      const unsigned char* sbt = smem + L.btslot_at(qb);
      const float2* tb = (const float2*)(sbt + 2 * L.b);
      const float4* mus = (const float4*)(sbt + 2 * L.b + L.t);
      const int nval = p1 - (p0 + s * kSfSC);
      if (nval >= kSfSC)
        gen(std::false_type{}, sa, tb, mus, kSfSC);
      else
        gen(std::true_type{}, sa, tb, mus, nval);
      fence_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&full_a[qa]);
      if (++qa == kSfA) {
        qa = 0;
        pha ^= 1;
      }
      if (++qb == kSfB) {
        qb = 0;
        phb ^= 1;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp < 8) {
    // every issuer's MMAs are complete (each issuer committed once at its end)
    bool w = true;
    for (int q = 0; q < kSfIssuers; q++) w = w && mbar_wait_abort(&dfull[q], 0, &abort_flag, p.tc_wait);
    w = __all_sync(kFull, w);
    tc_fence_after();
    const bool good = w && !abort_flag && nstage > 0;
    // warp w: tensor-memory lanes 32 (w & 3) .., column half w >> 2; the
    // accumulators of the issuers that had stages, added in order
    const int m = 32 * (warp & 3) + lane;
    const int c0 = (warp >> 2) * (NS / 2);
    const int nis = min(nstage, kSfIssuers);
    float* out = p.tc_part + (size_t)(chunk * p.tc_mt + mtile) * NS * 128;
    for (int cc = c0; cc < c0 + NS / 2; cc += 8) {
      float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int q = 0; q < nis; q++) {
        float v[8];
        tmem_ld8(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)q * acols + cc, v);
        tmem_wait_ld();
#pragma unroll
        for (int u = 0; u < 8; u++) acc[u] += v[u];
      }
#pragma unroll
      for (int u = 0; u < 8; u++) out[(size_t)(cc + u) * 128 + m] = good ? acc[u] : 0.f;
    }
    if (!w && lane == 0) atomicOr(p.err, kErrTcWait);
  }
  if (mtile == 0) {
    // FP64 moment sum of this chunk (surface term)
    const float4* gmu = (const float4*)p.s.mu;
    double m0 = 0, m1 = 0, m2 = 0;
    if (warp < kSfGenWarps)
      for (int q = p0 + tid; q < p1; q += 32 * kSfGenWarps) {
        const float4 mu = gmu[q];
        m0 += (double)mu.x;
        m1 += (double)mu.y;
        m2 += (double)mu.z;
      }
    m0 = warp_sum(m0);
    m1 = warp_sum(m1);
    m2 = warp_sum(m2);
    if (lane == 0 && warp < kSfGenWarps) {
      red[0][warp] = m0;
      red[1][warp] = m1;
      red[2][warp] = m2;
    }
    __syncthreads();
    if (tid < 3) {
      double s = 0;
      for (int w = 0; w < kSfGenWarps; w++) s += red[tid][w];
      p.musum_part[3 * chunk + tid] = s;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tmem, ncols);
}

__global__ void __launch_bounds__(kSfThreads) k_sf_tc(KParams p) { sf_tc_body(p, blockIdx.x, blockIdx.y); }
// Packed systems: one block per task (system, M tile + tc_mt x chunk).
__global__ void __launch_bounds__(kSfThreads) k_sf_tc_packed(const KParams* __restrict__ ps,
                                                            const Task* __restrict__ tk) {
  const Task t = tk[blockIdx.x];
  const KParams& p = ps[t.rep];
  const int mt = p.tc_mt;
  sf_tc_body(p, t.blk % mt, t.blk / mt);
}

// One element of the scatter operand image: hi at [t][0], lo at [t][1].
__device__ __forceinline__ void w_put(float* img, int kp, int row, int k, float x) {
  float h, l;
  tf32_split(x, h, l);
  const int o = cm_off(row, k, kp) >> 2;
  img[o] = h;
  img[kScCols * kp + o] = l;
}

// Block per (M tile, column q): 64 rows x G groups of chunks, the groups
// combined in a fixed order.  A single system (its chunks fill the GPU, 64 at
// N = 32768) takes 8 groups; packed batches take 2 (blocks of 128 threads, 16
// resident per SM: a small system has few chunks, which would leave most
// threads of a wider block idle, and a batch runs thousands of these blocks).  The chunk partials (FP32 tensor-memory sums of
// <= 512 particles) are added exactly: within a group with error-free FP32
// transformations (TwoSum: the running sum and its exact rounding errors;
// GB300's FP64 rate is a small fraction of FP32, so a conversion and an FP64
// addition per partial would cost more than the whole FP32 reduction), the
// group sum (sum + compensation) and the groups in FP64, as are S(n) = C_U +
// nx C_V and e(n) S(n); the W image is then split into its FP32 operands.
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float v) {
  const float t = s + v;
  const float bp = t - s;
  c += (s - (t - bp)) + (v - bp);  // the exact rounding error of s + v (Knuth)
  s = t;
}

constexpr int kRedGroups = 8, kRedGroupsPacked = 2;

template <bool FULL, int G>
__device__ __forceinline__ void sf_reduce_body(const KParams& p, int bx) {
  using L = ScatLayout<FULL>;
  __shared__ double red[G][4][64];  // [group][4 values][row]
  const int Q = 2 * p.kc + 1;
  const int mtile = bx / Q, q = bx - mtile * Q;
  const int rl = threadIdx.x & 63, grp = threadIdx.x >> 6;
  if (bx == 0 && threadIdx.x < 3) {
    double s = 0;
    for (int c = 0; c < p.tc_nchunk; c++) s += p.musum_part[3 * c + threadIdx.x];
    p.musum[threadIdx.x] = s;
  }
  const int NS = p.tc_ns;
  const size_t cstride = (size_t)p.tc_mt * NS * 128;
  const float* b = p.tc_part + (size_t)mtile * NS * 128;
  float su[4] = {0.f, 0.f, 0.f, 0.f}, cu[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
  for (int c = grp; c < p.tc_nchunk; c += G) {
    const float* bc = b + (size_t)c * cstride;
    two_sum_acc(su[0], cu[0], bc[(2 * q) * 128 + rl]);
    two_sum_acc(su[1], cu[1], bc[(2 * q + 1) * 128 + rl]);
    two_sum_acc(su[2], cu[2], bc[(2 * q) * 128 + 64 + rl]);
    two_sum_acc(su[3], cu[3], bc[(2 * q + 1) * 128 + 64 + rl]);
  }
#pragma unroll
  for (int v = 0; v < 4; v++) red[grp][v][rl] = (double)su[v] + (double)cu[v];
  __syncthreads();
  if (grp != 0) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int g = 0; g < G; g++)
#pragma unroll
    for (int v = 0; v < 4; v++) acc[v] += red[g][v][rl];
  const int r = mtile * 64 + rl;
  if (r >= p.tc_rows) return;
  const int kk = p.tc_kmap[r * Q + q];
  if (kk < 0) return;
  const double nxd = (double)(q - p.kc);
  const double srd = fma(nxd, acc[2], acc[0]), sid = fma(nxd, acc[3], acc[1]);
  p.S[kk] = make_double2(srd, sid);
  const double ed = p.ek[kk];
  const float er = (float)(ed * srd), ei = (float)(ed * sid);
  const float nx = (float)(q - p.kc);  // small integer: its powers below are exact
  const int tt = r / L::RT, sl = r - tt * L::RT;
  const int kp = p.tc_kp;
  float* img = p.tc_w + (size_t)tt * 2 * kScCols * kp;
  float f = 1.f;
#pragma unroll
  for (int pp = 0; pp < L::P; pp++) {
    // W_p = nx^p conj(e S): (wr, wi)
    const float wr = f * er, wi = -f * ei;
    const int col = L::ccol(sl, pp);
    w_put(img, kp, 2 * col, 2 * q, wr);
    w_put(img, kp, 2 * col, 2 * q + 1, -wi);
    w_put(img, kp, 2 * col + 1, 2 * q, wi);
    w_put(img, kp, 2 * col + 1, 2 * q + 1, wr);
    f *= nx;
  }
}

template <bool FULL>
__global__ void __launch_bounds__(64 * kRedGroups) k_sf_tc_reduce(KParams p) {
  sf_reduce_body<FULL, kRedGroups>(p, blockIdx.x);
}
// Packed systems: one block per task (system, M tile x column).
template <bool FULL>
__global__ void __launch_bounds__(64 * kRedGroupsPacked) k_sf_tc_reduce_packed(const KParams* __restrict__ ps,
                                                                             const Task* __restrict__ tk) {
  const Task t = tk[blockIdx.x];
  sf_reduce_body<FULL, kRedGroupsPacked>(ps[t.rep], t.blk);
}

// ---------------------------------------------------------------- scatter

// Roles (warps): 0-15 epilogue (warp w owns the tensor-memory lanes
// 32 (w & 3) .. = its particles and the quarter w >> 2 of each tile), 16 copy
// producer (bulk copies of W tiles into NST stages), 17 and 18 MMA issuers
// (tiles alternate between them, each into its own 128-column accumulator;
// two issuing threads keep the tensor cores busy with these small MMAs).
// The particles' X phases (the A operand, hi and lo) sit in tensor memory
// (columns [0, 2 kp)), the accumulators at columns 256 and 384.  An
// epilogue warp releases an accumulator as soon as it has loaded it.
template <bool FULL>
__device__ __forceinline__ void kscat_body(const KParams& p, int bx) {
  using L = ScatLayout<FULL>;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full_bar[kScMaxStages];  // W tile landed in a stage
  __shared__ __align__(8) uint64_t sfree_bar[kScMaxStages]; // the MMAs that read the stage are done
  __shared__ __align__(8) uint64_t dfull_bar[2];            // accumulator of issuer i complete
  __shared__ __align__(8) uint64_t dfree_bar[2];            // accumulator of issuer i loaded by the epilogue
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  const int kp = p.tc_kp, kc = p.kc, K1 = kc + 1, n = p.n, R = p.tc_rows, NT = p.tc_nt, NST = p.tc_nst;
  const int tbytes = 2 * kScCols * kp * 4;
  unsigned char* stage0 = smem;
  // row descriptors (kspace_tc_row_desc): ny, nz, offsets of Y(|ny|) and
  // Z(nz) in the phase table this block reads; the sign of ny conjugates Y
  const float4* __restrict__ rows_d = p.tc_rowd;
  // Y(|ny|), Z(nz) of the block's particles, [2 K1][128] (when p.tc_yz)
  float2* yz_s = (float2*)(stage0 + NST * tbytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool epi = warp < kScEpiWarps;
  const int quarter = warp & 3, cq = (warp >> 2) & 3;  // lane quarter, column quarter
  const int pl = 32 * quarter + lane;  // particle of this epilogue thread = tensor-memory lane
  const int i = bx * kScParticles + pl;
  const bool act = epi && i < n;
  const int ii = i < n ? i : n - 1;
  const float2* gtab = (const float2*)p.tab;

  if (tid == 0) {
    for (int q = 0; q < kScMaxStages; q++) {
      mbar_init(&full_bar[q], 1);
      mbar_init(&sfree_bar[q], 1);
    }
    for (int q = 0; q < 2; q++) {
      mbar_init(&dfull_bar[q], 1);
      mbar_init(&dfree_bar[q], kScEpiWarps);
    }
    mbar_init_fence();
    abort_flag = 0;
  }
  if (warp == 0) tmem_alloc(&tslot, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;
  if (epi) {
    if (p.tc_yz)
      for (int e = cq; e < 2 * K1; e += 4) yz_s[e * kScParticles + pl] = gtab[(size_t)(K1 + e) * n + ii];
    // A row of this particle into its tensor-memory lane: X(nx), nx = q - kc,
    // at k = 2q (Re), 2q + 1 (Im); hi at column k, lo at kp + k; the four
    // warps of a lane quarter write a quarter of the row's 4-column groups each
    const uint32_t lrow = tmem + ((uint32_t)(32 * quarter) << 16);
    const int ng = kp / 4, gq = (ng + 3) / 4;
    for (int c = cq * gq; c < min(ng, (cq + 1) * gq); c++) {
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
      float hi[4], lo[4];
#pragma unroll
      for (int u = 0; u < 4; u++) tf32_split(v[u], hi[u], lo[u]);
      tmem_st4(lrow + 4 * c, hi);
      tmem_st4(lrow + kp + 4 * c, lo);
    }
    tmem_wait_st();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  float b[3] = {0.f, 0.f, 0.f}, cb[3] = {0.f, 0.f, 0.f}, f[3] = {0.f, 0.f, 0.f}, cfr[3] = {0.f, 0.f, 0.f};
  const uint32_t dcol[2] = {256u, 384u};

  if (warp == kScEpiWarps) {
    // copy producer
    if (lane == 0) {
      bool ok = true;
      int issued = 0;
      for (int u = 0; u < NST && u < NT; u++) {
        mbar_expect_tx(&full_bar[u], tbytes);
        bulk_g2s(stage0 + u * tbytes, p.tc_w + (size_t)u * (tbytes / 4), tbytes, &full_bar[u]);
        issued = u + 1;
      }
      for (int t = 0; t + NST < NT && ok; t++) {
        // the stage of tile t takes tile t + NST once tile t's MMAs are done
        ok = mbar_wait_abort(&sfree_bar[t % NST], (t / NST) & 1, &abort_flag, p.tc_wait);
        if (!ok) break;
        const int u = t + NST;
        mbar_expect_tx(&full_bar[u % NST], tbytes);
        bulk_g2s(stage0 + (u % NST) * tbytes, p.tc_w + (size_t)u * (tbytes / 4), tbytes, &full_bar[u % NST]);
        issued = u + 1;
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(p.err, kErrTcWait);
      }
      // no copy may still be in flight at the exit: the last copy of each stage has landed
      for (int u = issued - NST > 0 ? issued - NST : 0; u < issued; u++)
        mbar_wait(&full_bar[u % NST], (u / NST) & 1, p.tc_wait);
    }
  } else if (warp > kScEpiWarps) {
    // MMA issuer 0 or 1: tiles t = is, is + 2, ...
    const int is = warp - kScEpiWarps - 1;
    if (lane == 0) {
      const uint32_t idesc = tc_idesc_tf32(128, kScCols);
      const uint32_t sbo = kp * 32;
      const uint32_t d = tmem + dcol[is];
      bool ok = true;
      int k = 0, last = -1;
      for (int t = is; t < NT && ok; t += 2, k++) {
        ok = mbar_wait_abort(&full_bar[t % NST], (t / NST) & 1, &abort_flag, p.tc_wait);
        if (ok && k >= 1) ok = mbar_wait_abort(&dfree_bar[is], (k - 1) & 1, &abort_flag, p.tc_wait);
        if (!ok) break;
        tc_fence_after();
        const uint64_t dbh = tc_desc(smem_u32(stage0 + (t % NST) * tbytes), 128, sbo);
        const uint64_t dbl = dbh + (uint64_t)((kScCols * kp * 4) >> 4);
#pragma unroll 2
        for (int ks = 0; ks < kp / 8; ks++) {
          const uint64_t o = 16 * ks;
          tc_mma_tf32_ta(d, tmem + 8 * ks, dbh + o, idesc, ks > 0);
          tc_mma_tf32_ta(d, tmem + 8 * ks, dbl + o, idesc, true);
          tc_mma_tf32_ta(d, tmem + kp + 8 * ks, dbh + o, idesc, true);
        }
        tc_commit(smem_u32(&dfull_bar[is]));
        tc_commit(smem_u32(&sfree_bar[t % NST]));
        last = k;
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(p.err, kErrTcWait);
      }
      if (last >= 0) mbar_wait(&dfull_bar[is], last & 1, p.tc_wait);  // this issuer's MMAs are done
    }
  } else {
    const float4 mu = act ? ((const float4*)p.s.mu)[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    auto kahan = [](float& s, float& c, float v) {
      const float y = v - c, t = s + y;
      c = (t - s) - y;
      s = t;
    };
    // P = Y(ny) Z(nz) of this particle for the rows of its quarter of tile t
    auto fetch = [&](int t, float2* P) {
#pragma unroll
      for (int sh = 0; sh < L::RQ; sh++) {
        const float4 d = __ldg(rows_d + t * L::RT + cq * L::RQ + sh);
        const int yo = __float_as_int(d.z), zo = __float_as_int(d.w);
        float2 y, z;
        if (p.tc_yz) {
          y = yz_s[yo + pl];
          z = yz_s[zo + pl];
        } else {
          y = gtab[yo + ii];
          z = gtab[zo + ii];
        }
        // conj Y for ny < 0: the sign bit of ny onto Im Y
        y.y = __int_as_float(__float_as_int(y.y) ^ (__float_as_int(d.x) & 0x80000000));
        P[sh] = make_float2(y.x * z.x - y.y * z.y, y.x * z.y + y.y * z.x);
      }
    };
    float2 Pc[L::RQ];
    if (NT > 0) fetch(0, Pc);
    for (int t = 0; t < NT; t++) {
      const int is = t & 1, k = t >> 1;
      float2 Pn[L::RQ];
      if (t + 1 < NT) fetch(t + 1, Pn);  // in flight during this tile's wait and arithmetic
      bool w = mbar_wait_abort(&dfull_bar[is], k & 1, &abort_flag, p.tc_wait);
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
      tmem_ld32(tmem + ((uint32_t)(32 * quarter) << 16) + dcol[is] + (uint32_t)(32 * cq), v);
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&dfree_bar[is]);
      float tb0 = 0.f, tb1 = 0.f, tb2 = 0.f, tf0 = 0.f, tf1 = 0.f, tf2 = 0.f;
#pragma unroll
      for (int sh = 0; sh < L::RQ; sh++) {
        {
          const float2 nn = __ldg((const float2*)(rows_d + t * L::RT + cq * L::RQ + sh));
          const float pr = Pc[sh].x, pi = Pc[sh].y;
          const float nyf = nn.x, nzf = nn.y;
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
#pragma unroll
      for (int sh = 0; sh < L::RQ; sh++) Pc[sh] = Pn[sh];
    }
  }
  tc_fence_before();
  __syncthreads();
  // the column quarters' sums of each particle, added in a fixed order; the
  // stage buffers are free now (every copy landed, every MMA completed)
  float* part = (float*)stage0;  // [3][6][kScParticles]
  if (epi && cq > 0) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
      part[((cq - 1) * 6 + a) * kScParticles + pl] = b[a] - cb[a];
      part[((cq - 1) * 6 + 3 + a) * kScParticles + pl] = f[a] - cfr[a];
    }
  }
  __syncthreads();
  if (act && cq == 0) {
    float sb[6];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      sb[a] = b[a] - cb[a];
      sb[3 + a] = f[a] - cfr[a];
    }
    for (int g = 0; g < 3; g++)
#pragma unroll
      for (int a = 0; a < 6; a++) sb[a] += part[(g * 6 + a) * kScParticles + pl];
    float* B = (float*)p.B;
    const float cfl = (float)p.cflux;
    B[i] = -cfl * sb[0];
    B[n + i] = -cfl * sb[1];
    B[2 * n + i] = -cfl * sb[2];
    if constexpr (FULL) {
      float* F = (float*)p.F;
      const float cfo = (float)p.cforce;
      F[i] = cfo * sb[3];
      F[n + i] = cfo * sb[4];
      F[2 * n + i] = cfo * sb[5];
    }
  }
  if (warp == 0) tmem_free(tmem, 512);
}

template <bool FULL>
__global__ void __launch_bounds__(kScThreads) k_kscat_tc(KParams p) {
  kscat_body<FULL>(p, blockIdx.x);
}
// Packed systems: one block per task (system, block of 128 particles).
template <bool FULL>
__global__ void __launch_bounds__(kScThreads) k_kscat_tc_packed(const KParams* __restrict__ ps,
                                                                 const Task* __restrict__ tk) {
  const Task t = tk[blockIdx.x];
  kscat_body<FULL>(ps[t.rep], t.blk);
}

// ------------------------------------------------------------ host side

static int rows_bound(int kc) { return (kc + 1) * (2 * kc + 1); }

bool kspace_tc_supported(int kc) {
  return kc >= 1 && kc <= kTcMaxKc && sf_smem(kc) <= kSmemLimit && scat_smem(kc, 2, rows_bound(kc)) <= kSmemLimit &&
         tc_ns(kc) <= 256;
}

int kspace_tc_max_kc() {
  int k = 0;
  for (int q = 1; q <= kTcMaxKc; q++)
    if (kspace_tc_supported(q)) k = q;
  return k;
}

TcShape kspace_tc_shape(int kc, int n, int rows, int nsm, int ring, int wave_mult) {
  TcShape s{};
  s.ns = tc_ns(kc);
  s.kp = tc_kp(kc);
  s.mt = (rows + 63) / 64;
  // the epilogue's Y, Z phases in shared memory when they fit beside two
  // stages (the epilogue, not the W-tile copies, bounds the scatter)
  s.yz = scat_smem(kc, 2, rows, true) <= kSmemLimit ? 1 : 0;
  // W-tile stages: a multiple of the two issuers, which alternate tiles and
  // wait on their tile's stage by parity (see sf_layout)
  s.nst = s.yz ? 2 : (scat_smem(kc, 4, rows) <= kSmemLimit ? 4 : 2);
  s.scat_smem = (int)scat_smem(kc, s.nst, rows, s.yz != 0);
  s.nt_full = (rows + ScatLayout<true>::RT - 1) / ScatLayout<true>::RT;
  s.nt_field = (rows + ScatLayout<false>::RT - 1) / ScatLayout<false>::RT;
  s.rt_full = ScatLayout<true>::RT;
  s.rt_field = ScatLayout<false>::RT;
  s.nsb = (n + kSfSC - 1) / kSfSC;
  const SfLayout sl = sf_layout(kc, ring);
  s.sfa = sl.na;
  s.sfb = sl.nb;
  // structure-factor grid: M tiles x chunks of <= kSfMaxChunk particles, the chunk
  // count filling whole waves of resident blocks (times `waves`: more, smaller
  // chunks, a tuning choice)
  int res = (int)((228 * 1024) / ((size_t)sl.bytes + 4096));
  res = std::max(1, std::min(res, 2));
  const long slots = (long)nsm * res;
  const long nch_min = std::max(1L, ((long)n + kSfMaxChunk - 1) / kSfMaxChunk);
  const long waves = std::max(1L, ((long)s.mt * nch_min + slots - 1) / slots) * std::max(1, std::min(wave_mult, 4));
  long nch = std::max(nch_min, waves * slots / (long)std::max(1, s.mt));
  nch = std::min<long>(nch, std::max(1L, ((long)n + kSfSC - 1) / kSfSC));
  s.chunk = (int)((((long)n + nch - 1) / nch + kSfSC - 1) / kSfSC * kSfSC);
  s.nchunk = (n + s.chunk - 1) / s.chunk;
  return s;
}

int kspace_tc_rows_pad(int R) { return scat_rows_pad(R); }

void kspace_tc_row_desc(const int2* rows, int R, int kc, int n, bool yz, float4* out) {
  const int K1 = kc + 1, ts = yz ? kScParticles : n;  // row stride of the phase table the scatter reads
  for (int r = 0; r < scat_rows_pad(R); r++) {
    const int2 rr = r < R ? rows[r] : make_int2(0, 0);
    const int ay = rr.x < 0 ? -rr.x : rr.x;
    const int yo = (yz ? ay : K1 + ay) * ts, zo = (yz ? K1 + rr.y : 2 * K1 + rr.y) * ts;
    float4 d;
    d.x = (float)rr.x;
    d.y = (float)rr.y;
    std::memcpy(&d.z, &yo, 4);
    std::memcpy(&d.w, &zo, 4);
    out[r] = d;
  }
}

size_t kspace_tc_image_floats(int kc, int nt) { return (size_t)nt * 2 * kScCols * tc_kp(kc); }
size_t kspace_tc_bimg_floats(int kc, int nsb) { return (size_t)nsb * tc_ns(kc) * kSfSK; }  // FP16 hi, lo
size_t kspace_tc_tblk_entries(int kc, int nsb) { return (size_t)nsb * 2 * (kc + 1) * kTabPad; }

int launch_kspace_tc_prep(cudaStream_t st, const KParams& p) {
  k_tc_prep<<<(p.n + kSfSC - 1) / kSfSC, 256, 0, st>>>(p);
  return 1;
}

size_t kspace_tc_sf_bytes(const TcShape& t, int kc) { return (size_t)SfLayout(t.ns, kc + 1, t.sfa, t.sfb).bytes; }

int launch_kspace_tc_prep_packed(cudaStream_t st, const KParams* ps, const Packed& prep) {
  if (!prep.n) return 0;
  k_tc_prep_packed<<<prep.n, 256, 0, st>>>(ps, prep.tasks);
  return 1;
}

int launch_kspace_tc_packed(cudaStream_t st, const KParams* ps, const Packed& sf, const Packed& red,
                            const Packed& sc, bool full, size_t sf_smem, size_t sc_smem) {
  if (!sf.n) return 0;
  cudaFuncSetAttribute(k_sf_tc_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sf_smem);
  k_sf_tc_packed<<<sf.n, kSfThreads, sf_smem, st>>>(ps, sf.tasks);
  if (full) {
    k_sf_tc_reduce_packed<true><<<red.n, 64 * kRedGroupsPacked, 0, st>>>(ps, red.tasks);
    cudaFuncSetAttribute(k_kscat_tc_packed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_smem);
    k_kscat_tc_packed<true><<<sc.n, kScThreads, sc_smem, st>>>(ps, sc.tasks);
  } else {
    k_sf_tc_reduce_packed<false><<<red.n, 64 * kRedGroupsPacked, 0, st>>>(ps, red.tasks);
    cudaFuncSetAttribute(k_kscat_tc_packed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_smem);
    k_kscat_tc_packed<false><<<sc.n, kScThreads, sc_smem, st>>>(ps, sc.tasks);
  }
  return 3;
}

int launch_kspace_tc(cudaStream_t st, const KParams& p, bool full, cudaEvent_t* ev) {
  const size_t sm1 = (size_t)SfLayout(p.tc_ns, p.kc + 1, p.tc_sfa, p.tc_sfb).bytes;
  cudaFuncSetAttribute(k_sf_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  k_sf_tc<<<dim3(p.tc_mt, p.tc_nchunk), kSfThreads, sm1, st>>>(p);
  if (ev) cudaEventRecordWithFlags(ev[0], st, cudaEventRecordExternal);
  const int nred = p.tc_mt * (2 * p.kc + 1);
  if (full)
    k_sf_tc_reduce<true><<<nred, 64 * kRedGroups, 0, st>>>(p);
  else
    k_sf_tc_reduce<false><<<nred, 64 * kRedGroups, 0, st>>>(p);
  if (ev) cudaEventRecordWithFlags(ev[1], st, cudaEventRecordExternal);
  const size_t sm2 = (size_t)p.tc_scat_smem;
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

// ------------------------------------------------------ bounded-wait probe

// The error path of a wait that gives up, on its own: one warp takes tensor
// memory, waits on an mbarrier (phase 0) that gets its arrival only when
// `arrive` is set, and when the wait gives up records kErrTcWait and still
// frees its tensor memory -- the steps of every wait in the kernels above.
// Tests run it with a short limit and no arrival (a barrier nothing
// signals), then check that the context reports the error and keeps working.
__global__ void __launch_bounds__(32) k_tc_wait_probe(int* err, int arrive, long long limit) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  const int lane = threadIdx.x;
  if (lane == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncwarp();
  tmem_alloc(&tslot, 32);
  tc_fence_before();
  __syncwarp();
  tc_fence_after();
  const uint32_t tmem = tslot;
  if (arrive && lane == 0) mbar_arrive(&bar);
  __syncwarp();
  const bool ok = mbar_wait(&bar, 0, limit);
  if (!ok && lane == 0) atomicOr(err, kErrTcWait);
  __syncwarp();
  tc_fence_before();
  tmem_free(tmem, 32);
}

int launch_tc_wait_probe(cudaStream_t st, int* err, int arrive, long long limit) {
  k_tc_wait_probe<<<1, 32, 0, st>>>(err, arrive, limit);
  return 1;
}

}  // namespace md
