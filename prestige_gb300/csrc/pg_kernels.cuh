// Kernel-ready parameter records and launchers shared by the .cu files of the library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_internal.cuh"

namespace pg {

// Arithmetic of the pair kernels.
enum Arith {
  ARITH_F64_EXACT = 0,  // IEEE double, oracle operation order (bit-exact)
  ARITH_F64_DF = 1,     // double-word arithmetic on the FP32 pipe (f64 tolerance)
  ARITH_F32_EXACT = 2,  // IEEE single, oracle operation order (bit-exact)
  ARITH_F32_FAST = 3,   // single precision with fused multiply-add
};

constexpr int kSphThreads = 128;     // default block size of the SPH kernels
constexpr int kSphMaxThreads = 256;  // largest block size of the list-based kernels
constexpr uint32_t kListTile = 32;  // slots per tile of the neighbour-list array
constexpr size_t kPackPad = 16;      // records allocated past the end of every sorted pack: the
                                     // list kernel's batched loads run up to kListBatch - 1 past
                                     // the last slot

// Stages of the SPH pair pass.
enum SphStage {
  SPH_RATES = 0,  // continuity and momentum rates of one state (pg_compute_rates)
  SPH_CONT = 1,   // continuity rate, then rho' = rho + dt C (first pass of a step)
  SPH_MOM = 2,    // momentum rate with rho', then v' and x' (second pass of a step)
};

// SPH constants of one system in one precision (formulas of the oracle's sph_consts).
template <class R>
struct SphC {
  R fa, fb, inv_h, four_h2, avk, eps_h2, B, inv_rho0, dt;
  R g[3];
};

// Double-word (hi, lo) copies of the constants for the f64 fast mode.
struct SphDF {
  float fa[2], fb[2], inv_h[2], four_h2[2], avk[2], eps_h2[2], B[2], inv_rho0[2];
  // F = c0 + c1 r + c2 / r, the cubic spline's (dW/dr)/r on each piece: q < 1 (near) and
  // 1 <= q < 2 (far), with q = r/h:  near c0 = -3 fa, c1 = 2.25 fa/h;  far c0 = -4 fb/h,
  // c1 = fb/h^2, c2 = 4 fb
  float near0[2], near1[2], far0[2], far1[2], far2[2];
  float h2;  // h^2: r^2 < h^2 selects the near piece
  float band;  // |r^2 - (2h)^2| below which the exact f64 test decides
};

struct SphK {
  GridK g;
  SphC<double> d;
  SphC<float> f;
  SphDF w;
  float two_h_f;
  double pos_pad;                        // double-word mode: 8h, packed positions are x - min + pos_pad
  double avk_alpha;                      // d avk / d alpha = -2 c0 h (adjoint)
  uint32_t id_begin, id_end, fluid_end;  // global ids; ids >= fluid_end are fixed wall particles
  int gamma;
};

struct SphArgs {
  const SphK* sys;           // per system (device)
  const uint32_t* sys_of_id; // null for a single system
  uint32_t n;
  int dim, reach;
  const uint32_t* sorted_cell;
  const uint32_t* sorted_id;
  const uint32_t* cell_start;
  void* s[8];                // sorted packed arrays (layout per arithmetic mode)
  void* pos;                 // canonical state, id order
  void* vel;
  void* rho;
  void* mass;
  void* acc;                 // optional rates output, id order
  void* drho;
  unsigned long long* posmin;  // double-word mode: per system and dimension ([3 sys + d]) the minimum
                               // position of the step, order-preserving integer code (hash_kernel)
  void* lam[5];              // adjoint (pg_adjoint.cu): lambda_x, lambda_v, lambda_rho, dL/dalpha and
                             // dL/dB partial sums, all id order
  uint32_t* nlist;           // neighbour lists in tiles of kListTile slots: entry q of slot k at
                             // nlist[(k / 32) * cap * 32 + q * 32 + k % 32] (q < min(nlen[k], cap))
  uint32_t* nlen;            // neighbours of slot k that passed the prefilter (may exceed cap)
  uint32_t* nresume;         // (row, slot) where the walk continues when nlen[k] > cap
  void* fcache;              // per list entry, same tiling as nlist: double-word mode {m_j F, u} (hi, lo);
                             // IEEE double: planes of F, w and r^2 + eps h^2
  uint32_t cap;
  uint32_t k_begin, k_end;   // sorted slots handled by the list and pair kernels (k_begin a multiple
                             // of the block size; the whole system is [0, n))
  unsigned* err;             // device error word (ERR_* bits)
  int integrate;
};

int launch_sph_gather(cudaStream_t st, const SphArgs& a, int arith);
int launch_sph_repack_rho(cudaStream_t st, const SphArgs& a, int arith);  // packed rho', P' from rho
// Neighbour lists for the list-based passes (stage passes read a.nlist / a.nlen / a.nresume).
// block: threads per block (multiple of 32, <= kSphMaxThreads).
int launch_sph_list(cudaStream_t st, const SphArgs& a, int arith, int grid, int block);
// lanes: threads per slot of the continuity and momentum passes (1, 2 or 4: 32, 16 or 8
// particles per warp); only the tolerance-based modes (double-word f64, contracted f32) take
// more than one, the others run 1 (sph_pass_lanes gives the count a pass actually uses).
int launch_sph_list_pass(cudaStream_t st, const SphArgs& a, int arith, int stage, int grid, int block,
                         int lanes = 1);
int sph_pass_lanes(int arith, int stage, int lanes);
int sph_list_regs(int arith, int dim, int stage, int lanes = 1);  // registers per thread of a list kernel (stage < 0) or pass
int sph_list_occupancy(int arith, int dim, int stage, int block, int lanes = 1);  // stage < 0: the list kernel
// The list kernel with an explicit FP32 prefilter-position pack a.s[pf_index] (conservative test).
int launch_sph_list_pf(cudaStream_t st, const SphArgs& a, int pf_index, int grid, int block);
// The IEEE f64 step with each neighbour pair evaluated once (pg_sph_sym.cu), over complete lists:
// part 0 and 1 the continuity pass (pair values, then the sums, rho' and the {rho', P'} pack),
// part 2 and 3 the momentum pass (pair values, then the sums and the update).  a.fcache holds
// sph_sym_entry_bytes() per list entry.
// split > 0 (part 0 only): the lists of the slots from split on may still be being built; the
// launch with second == 0 takes the slots whose partners all lie below split, second == 1 the rest.
int launch_sph_sym(cudaStream_t st, const SphArgs& a, int part, int block, uint32_t split = 0, int second = 0);
size_t sph_sym_entry_bytes();

// Adjoint of one SPH step (pg_adjoint.cu).  s[0..4] hold the slot-ordered packs written by
// launch_adjoint_prep; pos/vel/rho/mass are the state before the step (id order).
// fp32: mixed-precision packs and pair terms (double-precision adjoint accumulators).
int launch_adjoint_prep(cudaStream_t st, const SphArgs& a, bool fp32);
int launch_adjoint_pass(cudaStream_t st, const SphArgs& a, int stage, int grid, bool fp32);
int adjoint_pass_occupancy(int dim, int stage, bool fp32);
int adjoint_pf_index(bool fp32);
// The FP64 adjoint passes with each pair evaluated once (pg_adjoint_sym.cu), over exact lists
// (launch_sph_list_exact): part 0 the mirror indices, 1, 2 the momentum adjoint, 3, 4 the
// continuity adjoint.
// a.fcache: adjoint_sym_entry_bytes() per list entry; a.s[6]: adjoint_sym_slot_bytes() per slot.
int launch_adjoint_sym(cudaStream_t st, const SphArgs& a, int part);
size_t adjoint_sym_entry_bytes();
size_t adjoint_sym_slot_bytes();
// The list kernel with the f64 test of the exact neighbours on the double4 positions a.s[0] and
// the FP32 prefilter positions a.s[pf_index].
int launch_sph_list_exact(cudaStream_t st, const SphArgs& a, int pf_index, int grid, int block);
// Bytes per particle of the sorted packed arrays s[0..5] for an arithmetic mode.
void sph_sorted_layout(int arith, size_t sizes[6]);

// ---------------------------------------------------------------------------------------
// Neighbour utilities (counts, CSR lists, the eq1 gather) on the sorted positions.
// ---------------------------------------------------------------------------------------
struct NbrArgs {
  const GridK* grid;          // per system (device)
  const uint32_t* sys_of_id;  // null for a single system
  uint32_t n;
  int dim, reach, f64;
  const uint32_t* sorted_cell;
  const uint32_t* sorted_id;
  const uint32_t* cell_start;
  const void* spos;           // sorted positions: double4_32a or float4 (x, y, z, 0)
};

int launch_sorted_positions(cudaStream_t st, const NbrArgs& a, const void* pos, void* spos);
int launch_neighbor_counts(cudaStream_t st, const NbrArgs& a, uint32_t* counts_by_id);
int launch_neighbor_list(cudaStream_t st, const NbrArgs& a, const uint32_t* offs_by_id, uint32_t* nbr);
int launch_gather_sum(cudaStream_t st, const NbrArgs& a, const double* src_sorted, double* dst_by_id);
int launch_gather_field(cudaStream_t st, const uint32_t* sorted_id, uint32_t n, const double* src, double* out);

// ---------------------------------------------------------------------------------------
// DEM.
// ---------------------------------------------------------------------------------------
struct DemK {
  GridK g;
  double kn, kt, mu, dt, gcoef;
  double grav[3], wall_lo[3], wall_hi[3];
  float wall_lo_f[3], wall_hi_f[3];  // FP32 copies for the wall screen
  int capacity;
  int dt_finite;
};

struct DemArgs {
  const DemK* K;  // device
  uint32_t n;
  int reach;
  const uint32_t* sorted_cell;
  const uint32_t* sorted_id;
  const uint32_t* cell_start;
  double4_32a* sA;  // x, y, z, r
  double4_32a* sB;  // vx, vy, vz, m
  double4_32a* sW;  // wx, wy, wz, 0
  float4* sF;       // x, y, z, r rounded to FP32 (conservative candidate prefilter)
  double* pos;
  double* vel;
  double* omega;
  const double* radius;
  const double* mass;
  const uint32_t* hpid_old;
  const double* hxi_old;
  uint32_t* hpid_new;
  double* hxi_new;
  unsigned long long* contacts;
  unsigned* err;
};

int launch_dem_gather(cudaStream_t st, const DemArgs& a);
int launch_dem_pass(cudaStream_t st, const DemArgs& a);

}  // namespace pg
