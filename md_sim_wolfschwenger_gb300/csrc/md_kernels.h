// md_kernels.h -- host-side launch wrappers of the device kernels.  Each
// returns the number of kernel launches it issued on the stream.
//
// Two forms per kernel: one system (parameters by value), and packed: one
// grid over several systems, whose parameters sit in device arrays indexed
// by replica and whose blocks are listed in a task table (Task, built by the
// host from the per-system block counts below).  Packed launches exist for
// the mixed-precision path.
#pragma once
#include "md_common.cuh"

namespace md {

// Task table of one packed launch (device memory) and its length = grid size.
struct Packed {
  const Task* tasks;
  int n;
  WorkQ* wq;  // work queue of the persistent launches over this table (zeroed)
};

// Grid of a persistent packed launch: the blocks that one wave of kernel
// `fn` keeps resident (occupancy x SMs), at most ntask; its blocks stride
// over the task table.
int persistent_grid(const void* fn, int threads, size_t smem, int ntask);

// Blocks of one system per kernel shape (task-table construction).
int cell_blocks(int n);                 // cell assign/scatter/fill, integrator
int cell_sort_blocks(const CellGrid& g);
int real_blocks(int n);                 // real space and neighbour list
int real_pass_blocks(int n);            // real-space passes without coating (4-warp blocks)
int phase_blocks(int n);
int sk_blocks(const KParams& p);
// Threads (segments) per structure-factor block, and how many such blocks
// one SM holds at once for kc.
int sk_threads();
int sk_resident_blocks(int kc, bool fp64);
int skred_blocks(const KParams& p);
int scatter_blocks(const KParams& p, int np);
int int_blocks(int n);
int int_blocks_one(int n);        // single-system Heun launches (128-thread blocks)

// Step start: decides whether this step rebuilds the cell order and the
// neighbour list (host request, or a particle moved more than half_skin).
int launch_step_begin(cudaStream_t st, StepFlags* flags, double half_skin);
// anyrb: the batch's word "some system rebuilds its lists this step" (set here,
// read by the packed list kernels, cleared by launch_obs_packed's kernel)
int launch_step_begin_packed(cudaStream_t st, const CellParams* ps, int R, unsigned* anyrb);
// Raises the displacement since the last build after new positions arrived.
int launch_disp_check(cudaStream_t st, int n, const double* pos, const double* xbuild, double L, StepFlags* flags);
// State in from / out to host buffers the device addresses directly
// (device-side addresses of page-locked mapped memory); state_in also
// raises maxdisp against xbuild when it is not null.
int launch_state_in(cudaStream_t st, int n, const double* hpos, const double* hmm, const double* hea, double* pos,
                    double* mm, double* ea, const double* xbuild, double L, StepFlags* flags);
int launch_state_out(cudaStream_t st, int n, const double* pos, const double* mm, const double* ea, double* hpos,
                     double* hmm, double* hea);
// Cell order (skipped unless the step rebuilds) and the sorted views.
int launch_cells(cudaStream_t st, const CellParams& p, bool fp64);
int launch_cells_packed(cudaStream_t st, const CellParams* ps, int R, const Packed& n256, const Packed& sort,
                        const unsigned* anyrb);
// Neighbour list within rc + skin (count, scan, fill; skipped unless rebuilding).
int launch_nbr(cudaStream_t st, const RealParams& p, StepFlags* flags, bool fp64);
int launch_nbr_packed(cudaStream_t st, const RealParams* ps, int R, const Packed& real, const unsigned* anyrb);
int launch_set_mu(cudaStream_t st, int n, const double* mm, const double* magMom_u, const double* rMag_u,
                  const SortedView& s, bool fp64);

// Real space: full (field + force + pressure + overlap) or field only.
int launch_real(cudaStream_t st, const RealParams& p, bool full, bool fp64);
// pass: the 4-warp-block table (real_pass_blocks), used unless full && coat
int launch_real_packed(cudaStream_t st, const RealParams* ps, const Packed& real, const Packed& pass, bool full,
                       bool coat);

// k space: structure factor partials, reduction, scatter (full or field only).
// ev (optional): two events recorded after the structure factor and after
// the reduction.
int launch_kspace(cudaStream_t st, const KParams& p, bool full, bool fp64, cudaEvent_t* ev = nullptr);
// Packed k space; kcmax bounds the shared-memory tables, np = particles per
// scatter block (scatter_particles(kcmax)).
int launch_kspace_packed(cudaStream_t st, const KParams* ps, const Packed& sk, const Packed& red, const Packed& sc,
                         bool full, int kcmax, int np);
// Tensor-core k space (mixed path, md_ktc.cu): same sums, as matrix
// products over k rows.  Shape of the launches for kc, N particles, R k rows.
struct TcShape {
  int ns, kp, mt, nst;          // structure-factor N, scatter K, M tiles, scatter stages
  int nt_full, nt_field;        // scatter tiles (field + force, field only)
  int rt_full, rt_field;        // k rows per scatter tile
  int chunk, nchunk;            // structure-factor particle chunks
  int nsb;                      // structure-factor stages of 32 particles (per-step operand images)
  int sfa, sfb;                 // structure-factor ring slots (generated, copied)
  int scat_smem;                // dynamic shared memory of the scatter
  int yz;                       // scatter keeps the Y, Z phases in shared memory
};
bool kspace_tc_supported(int kc);
int kspace_tc_max_kc();  // largest supported kc
// ring: structure-factor ring option (-1: the deepest that fits); waves:
// multiplier of the wave-filling chunk count (1 .. 4).
TcShape kspace_tc_shape(int kc, int n, int rows, int nsm, int ring = -1, int waves = 1);
int kspace_tc_ring_options(int kc, int* opts_out, int cap);
size_t kspace_tc_image_floats(int kc, int nt);  // scatter operand image of nt tiles
// Scatter row descriptors: R rows padded to whole tiles of both shapes;
// (ny, nz, Y offset, Z offset bits) per row into out[kspace_tc_rows_pad(R)],
// offsets into the block's Y, Z copy (yz) or the global phase table.
int kspace_tc_rows_pad(int R);
void kspace_tc_row_desc(const int2* rows, int R, int kc, int n, bool yz, float4* out);
size_t kspace_tc_bimg_floats(int kc, int nsb);   // per-step X operand tiles
size_t kspace_tc_tblk_entries(int kc, int nsb);  // per-step Y, Z blocks (float2)
// Per-step operand images (after the phase tables), then per evaluation.
int launch_kspace_tc_prep(cudaStream_t st, const KParams& p);
int launch_kspace_tc(cudaStream_t st, const KParams& p, bool full, cudaEvent_t* ev = nullptr);
// Packed systems on the tensor cores: per-step operand prep (after the phase
// tables), and structure factor + reduction + scatter of one evaluation;
// task tables with one block per task, dynamic shared memory the largest of
// the packed systems' (kspace_tc_sf_bytes, TcShape::scat_smem).
size_t kspace_tc_sf_bytes(const TcShape& t, int kc);
int launch_kspace_tc_prep_packed(cudaStream_t st, const KParams* ps, const Packed& prep);
int launch_kspace_tc_packed(cudaStream_t st, const KParams* ps, const Packed& sf, const Packed& red,
                            const Packed& sc, bool full, size_t sf_smem, size_t sc_smem);
// One warp waits on an mbarrier that gets an arrival only when `arrive` is
// set; a wait that gives up after `limit` cycles sets kErrTcWait in *err.
int launch_tc_wait_probe(cudaStream_t st, int* err, int arrive, long long limit);
// Per-particle phase tables (once per step; positions are frozen across the
// two Heun stages).
int launch_phase_tables(cudaStream_t st, const KParams& p, bool fp64);
int launch_phase_tables_packed(cudaStream_t st, const KParams* ps, const Packed& phase);
// FP32 FMA-chain calibration: returns FLOPs issued by one launch.
double launch_fma_calibration(cudaStream_t st, float* out, int blocks, int threads);
size_t kscatter_smem(int kc, bool fp64);
size_t ksf_smem(int kc, bool fp64);
int scatter_particles(int kc, bool fp64);

// Integrator.
int launch_heun1(cudaStream_t st, const IntParams& p, bool fp64);
int launch_obs(cudaStream_t st, const ObsParams& p);
// Stage 2 with the step records (k_obs) fused: done = a zeroed block counter.
int launch_heun2_obs(cudaStream_t st, const IntParams& p, const ObsParams& o, unsigned* done, bool fp64);
int launch_heun1_packed(cudaStream_t st, const IntParams* ps, const Packed& n256);
int launch_heun2_packed(cudaStream_t st, const IntParams* ps, const Packed& n256);
int launch_obs_packed(cudaStream_t st, const ObsParams* ps, int R, unsigned* anyrb);
// B, F in SI (orig order, double) from the stage outputs; optional overlap push.
// Real-space field and force alone of the last full evaluation (test hook).
int launch_real_part(cudaStream_t st, const IntParams& p, double* Bout, double* Fout, bool fp64);
// Adaptive Runge-Kutta stage / accept kernels (md_integrate.cu).
int launch_rk_stage(cudaStream_t st, const RKStage& q, bool fp64);
int launch_rk_accept(cudaStream_t st, const RKStage& q, bool fp64);
int launch_combine(cudaStream_t st, const IntParams& p, double* Bout, double* Fout, int apply_overlap,
                   bool fp64);

}  // namespace md
