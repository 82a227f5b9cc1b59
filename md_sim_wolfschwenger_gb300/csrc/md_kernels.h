// md_kernels.h -- host-side launch wrappers of the device kernels.  Each
// returns the number of kernel launches it issued on the stream.
#pragma once
#include "md_common.cuh"

namespace md {

// Step start: decides whether this step rebuilds the cell order and the
// neighbour list (host request, or a particle moved more than half_skin).
int launch_step_begin(cudaStream_t st, StepFlags* flags, double half_skin);
// Raises the displacement since the last build after new positions arrived.
int launch_disp_check(cudaStream_t st, int n, const double* pos, const double* xbuild, double L, StepFlags* flags);
// Cell order (skipped unless the step rebuilds) and the sorted views.
int launch_cells(cudaStream_t st, int n, const double* pos, const double* mm, const double* magMom_u,
                 const double* rMag_u, double L, const CellGrid& g, int* cellOf, int* count, int* tmp,
                 const SortedView& s, bool fp64, double* xbuild, const StepFlags* flags);
// Neighbour list within rc + skin (count, scan, fill; skipped unless rebuilding).
int launch_nbr(cudaStream_t st, const RealParams& p, StepFlags* flags, bool fp64);
int launch_set_mu(cudaStream_t st, int n, const double* mm, const double* magMom_u, const double* rMag_u,
                  const SortedView& s, bool fp64);

// Real space: full (field + force + pressure + overlap) or field only.
int real_blocks(int n);
int launch_real(cudaStream_t st, const RealParams& p, bool full, bool fp64);

// k space: structure factor partials, reduction, scatter (full or field only).
// ev (optional): two events recorded after the structure factor and after
// the reduction.
int launch_kspace(cudaStream_t st, const KParams& p, bool full, bool fp64, cudaEvent_t* ev = nullptr);
// Per-particle phase tables (once per step; positions are frozen across the
// two Heun stages).
int launch_phase_tables(cudaStream_t st, const KParams& p, bool fp64);
// FP32 FMA-chain calibration: returns FLOPs issued by one launch.
double launch_fma_calibration(cudaStream_t st, float* out, int blocks, int threads);
size_t kscatter_smem(int kc, bool fp64);
size_t ksf_smem(int kc, bool fp64);

// Integrator.
int int_blocks(int n);
int launch_heun1(cudaStream_t st, const IntParams& p, bool fp64);
int launch_heun2(cudaStream_t st, const IntParams& p, bool fp64);
int launch_obs(cudaStream_t st, const ObsParams& p);
// B, F in SI (orig order, double) from the stage outputs; optional overlap push.
int launch_combine(cudaStream_t st, const IntParams& p, double* Bout, double* Fout, int apply_overlap,
                   bool fp64);

}  // namespace md
