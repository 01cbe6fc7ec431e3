// The handle behind the opaque `pg_system*` of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "pg_internal.cuh"
#include "pg_kernels.cuh"

struct pg_adjoint;  // checkpointed adjoint state (pg_adjoint.cu)

struct pg_system {
  // configuration
  pg_config cfg;                   // system 0 (shared fields of a batch)
  std::vector<pg_config> cfgs;     // one per system
  std::vector<size_t> id_begin;    // n_systems + 1 entries
  int model = PG_MODEL_SPH;
  int dim = 3;
  int f64 = 1;
  int arith = 0;
  size_t n = 0;
  int nsys = 1;
  cudaStream_t stream = nullptr;

  // grids and per-system tables (device copies)
  std::vector<pg::Grid> grids;
  uint64_t ncells = 0;
  pg::DevBuf gridk;      // GridK[nsys]
  pg::DevBuf sys_of_id;  // u32[n] (batched handles only)
  pg::DevBuf sphk;       // SphK[nsys]
  pg::DevBuf demk;       // DemK

  // canonical state, particle-id order
  pg::DevBuf pos, vel, rho, mass;  // SPH: system precision; DEM: double
  pg::DevBuf omega, radius;        // DEM
  pg::DevBuf acc, drho;            // rates output (pg_compute_rates)
  std::map<std::string, std::unique_ptr<pg::DevBuf>> user;  // user scalar fields (double)
  std::map<std::string, std::unique_ptr<pg::DevBuf>> snapshots;  // pre-call copies (pg_run_equations)

  // neighbour search and sorted copies
  pg::NbrWork nw;
  bool nbr_valid = false;
  bool stage_pending = false;  // pg_step_stage(0) ran; pg_step_stage(1) may follow
  pg::DevBuf sorted[6];
  pg::DevBuf spos;
  pg::DevBuf tmp, tmp2, tmp3, tmp4;
  int pass_grid[3] = {0, 0, 0};  // per SphStage
  int list_grid = 0;
  int block = 128;               // threads per block of the list-based SPH kernels
  int block_mom = 0;             // threads per block of the momentum pass (0: block)
  int lanes = 1;                 // threads per slot of the continuity and momentum passes (32 / particles per warp)
  int list_cap = 128;            // neighbour-list slots per particle
  // overlap of the continuity pass over slots [0, split) with the list kernel over [split, n) on
  // the auxiliary stream (split 0: off); reduced persistent grids let both kernels share the SMs
  uint32_t ov_split = 0;
  int ov_pass_grid = 0, ov_list_grid = 0;
  cudaStream_t aux = nullptr;
  cudaEvent_t ov_ev[2] = {nullptr, nullptr};
  pg::DevBuf nlist, nlen, nresume;
  pg::DevBuf fcache;             // f64 modes: pair values per list entry (continuity -> momentum)
  pg::DevBuf posmin;             // 3 x u64, double-word mode (pos_min_kernel)

  // DEM contact history, id order, double buffered
  pg::DevBuf hpid[2], hxi[2];
  int hcur = 0;
  pg::DevBuf contacts;  // unsigned long long

  // device error word
  pg::DevBuf err;

  // asynchronous host I/O (pg_set_field_async / pg_get_field_async): per field a staging buffer
  // for inputs and a snapshot buffer for outputs, one copy stream per direction
  struct IoSlot {
    pg::DevBuf stage, snap;
    size_t in_bytes = 0;
    bool pending = false;  // staged input not yet moved into the field
    cudaEvent_t in_ready = nullptr, in_free = nullptr, snap_ready = nullptr, snap_free = nullptr;
  };
  std::map<std::string, IoSlot> io;
  cudaStream_t io_in = nullptr, io_out = nullptr;

  // CUDA graph of one step (DEM: one per history parity)
  bool graph_enabled = false;
  int list_arith = -1;  // arithmetic mode of the pair lists in nlist/nlen (-1: none built yet)
  cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};

  // step timing (pg_timing_enable): 4 events per step, consumed by pg_timing_read
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<cudaEvent_t> ev_pending;
  pg_timing tacc;
  long long launches = 0;  // kernels enqueued by this handle

  // differentiable runs
  pg_adjoint* adj = nullptr;
  size_t adjoint_bytes() const;

  ~pg_system();
};

namespace pg {
size_t pg_elem_bytes(const pg_system* s);
int ensure_sorted_buffers(pg_system* s);
SphArgs sph_args(pg_system* s, int integrate, bool rates);
int enqueue_neighbors(pg_system* s);
int enqueue_sph_step(pg_system* s, bool rates, int integrate, cudaEvent_t* ev);
int enqueue_sph_front(pg_system* s, cudaEvent_t* ev);
int enqueue_sph_momentum(pg_system* s, cudaEvent_t* ev);
long long neighbor_launches(const pg_system* s);
int sync_and_check(pg_system* s);
int choose_pass_grid(pg_system* s);
int retune_sph(pg_system* s, double mult, int f64_mode, int block);
int mom_block(const pg_system* s);
int set_momentum_block(pg_system* s, int block);
int set_pass_lanes(pg_system* s, int lanes);
int enqueue_step(pg_system* s);
int apply_io_inputs(pg_system* s);
void drop_graphs(pg_system* s);
int capture_graphs(pg_system* s);
void destroy_adjoint(pg_system* s);
}  // namespace pg
