// Internal declarations of the GB300 (sm_103a) particle library.
//
// Data layout in HBM (one handle = one particle system, or a batch of independent systems
// concatenated in id order):
//   canonical state, particle-id order   pos[n*dim], vel[n*dim], rho[n], mass[n]   (SPH)
//                                        pos, vel, omega[n*3], radius[n], mass[n]  (DEM)
//   neighbour search, every step         cell of each id -> stable LSD radix sort by cell
//                                        -> sorted_cell[k], sorted_id[k] (slot k)
//                                        cell_start[c], n_cells + 1 entries
//   sorted packed copies, slot order     read by the pair kernels (coalesced, shared in L1)
// The pair kernels read only the sorted copies and write the canonical entries of their own
// particle, so one launch holds both the force loop and the integrator.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/prestige_gpu.h"

namespace pg {

// ---------------------------------------------------------------------------------------
// Errors: a thread-local message plus an integer status.
// ---------------------------------------------------------------------------------------
void set_error(const char* fmt, ...);
void clear_error();
const char* last_error();

#define PG_CUDA_TRY(expr)                                                                            \
  do {                                                                                               \
    cudaError_t e_ = (expr);                                                                         \
    if (e_ != cudaSuccess) {                                                                         \
      ::pg::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__);   \
      return e_ == cudaErrorMemoryAllocation ? PG_ENOMEM : PG_ECUDA;                                 \
    }                                                                                                \
  } while (0)

#define PG_TRY(expr)            \
  do {                          \
    int s_ = (expr);            \
    if (s_ != PG_OK) return s_; \
  } while (0)

// Device error word bits (set with atomicOr by kernels, read at synchronisation points).
enum : unsigned {
  ERR_CONTACT_OVERFLOW = 1u,  // DEM: a particle had more contacts than history slots
};

// ---------------------------------------------------------------------------------------
// Owned device buffer.  Allocated at set-up only, never inside a step, so a step can be
// captured into a CUDA graph.
// ---------------------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release();
  int ensure(size_t nbytes);  // grow to at least nbytes (contents undefined after growth)
  template <class T> T* as() const { return (T*)p; }
};

// ---------------------------------------------------------------------------------------
// Cell grid.  Cell side s = mult * support * (1 + 2^-20); the inflation keeps every pair
// closer than `support` within `reach` cells after rounding.  Cell index
// c = (cz * ny + cy) * nx + cx with c_d = clamp(floor((x_d - lo_d) * inv), 0, n_d - 1),
// evaluated as one IEEE subtraction then one multiplication in the system precision.
// Clamping is monotone, so particles outside the box still find every neighbour.
// ---------------------------------------------------------------------------------------
struct Grid {
  int dim = 3;
  double lo[3] = {0, 0, 0};
  double cell = 1.0, inv = 1.0, support = 1.0;
  int n[3] = {1, 1, 1};
  int reach = 1;
  uint64_t ncells() const { return (uint64_t)n[0] * n[1] * n[2]; }
};
int make_grid(int dim, const double lo[3], const double hi[3], double support, double mult, Grid* g);

// Kernel-side copy of a grid.
struct GridK {
  double lo[3];
  double inv;
  double support;
  float lof[3];
  float invf;
  float support_f;
  int nx, ny, nz;
  int reach;
  int dim;
  uint32_t cell_base;  // added to every cell index (batched systems)
};
GridK grid_k(const Grid& g, uint32_t cell_base);

// ---------------------------------------------------------------------------------------
// Neighbour-search workspace: stable LSD radix sort of (cell, id) and the cell table.
// ---------------------------------------------------------------------------------------
struct NbrWork {
  size_t n = 0;
  uint64_t ncells = 0;
  int passes = 0;
  int tiles = 0;
  int items = 16;  // keys per thread of the radix kernels (tiles of 256 * items keys)
  DevBuf keys[2], vals[2];  // u32
  DevBuf hist;              // u32 [256 * tiles]
  DevBuf digit_total;       // u32 [256]
  DevBuf cell_start;        // u32 [ncells + 1]
  uint32_t* sorted_cell = nullptr;
  uint32_t* sorted_id = nullptr;
  int init(size_t n, uint64_t ncells);
  size_t bytes() const;
};

// Cell key and id of every particle (id order) into w.keys[0] / w.vals[0].
// posmin (optional, f64 positions only): per system and dimension ([3 sys + d]) the minimum
// position, as ordered_code values, folded in with atomicMin (the caller presets it to all ones).
int launch_hash(cudaStream_t st, const GridK* grid_dev, const uint32_t* sys_of_id, int f64, int dim,
                const void* pos, size_t n, uint32_t* keys, uint32_t* vals, unsigned long long* posmin = nullptr);

// Order-preserving map of doubles to unsigned 64-bit integers (and back), for atomicMin.
__device__ __forceinline__ unsigned long long ordered_code(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ordered_value(unsigned long long u) {
  return __longlong_as_double((long long)((u >> 63) ? (u & 0x7fffffffffffffffull) : ~u));
}
// Sort (cell, id) pairs already in keys[0]/vals[0] and build cell_start.
int sort_and_table(cudaStream_t st, NbrWork& w);
// Exclusive scan of m u32 values into out[0..m] (out[m] = total).  tmp: scan_tmp_words(m).
size_t scan_tmp_words(size_t m);
int launch_exclusive_scan(cudaStream_t st, const uint32_t* in, uint32_t* out, size_t m, uint32_t* tmp);

}  // namespace pg
