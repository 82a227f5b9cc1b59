// md_types.h -- plain structs shared by host code and kernels.
#pragma once

namespace md {

// Cell grid of the real-space neighbour search (cubic box).
struct CellGrid {
  int ncx;     // cells per box edge
  int ncell;   // ncx^3
  int reach;   // stencil half-width m in cells; 0 => all pairs (ncx == 1)
};

// One row segment of k vectors: (nx0 + t, ny, nz) for t < len.  len is a
// multiple of 4; the padding k's carry e(k) = 0.
struct KSeg {
  int nx0, ny, nz, len;
};

// k vectors per shared-memory chunk of the k-space scatter.
constexpr int kKChunk = 512;
// Longest k-row segment of the scatter (rows longer than this are split
// evenly); the structure factor uses segments of at most 16.
constexpr int kScatSeg = 64;
// Thread partitions of the k-space scatter: each particle's k range is split
// over this many threads (by chunk), reduced in a fixed order.
constexpr int kScatterParts = 4;

}  // namespace md
