// prestige.hpp -- C++ host layer over the C ABI of the GB300 particle library.
//
// It restates, in C++, the interface the reference exposes to its users (dineshadepu/prestige):
//   EquationIR            prestige/src/equations/ir.rs:3-14     {name, reads, writes, body}
//   equation()            prestige_macros/src/lib.rs:8-133      what #[equation] records: the
//                         slices a pairwise body reads and writes (the SliceVisitor rules)
//   FusedEquations, fuse  prestige/src/equations/fuse.rs:4-40   union of reads/writes, bodies in order
//   generate_simple_cpu   prestige/src/codegen/simple_cpu.rs:3-22  the all-pairs loop text
//   debug_equation        prestige/src/equations/debug.rs:3-22
// and adds the GPU backend the reference does not have: run_gpu() executes a fused set on a
// System (a device-resident particle handle) with j restricted to the neighbour set: the
// built-in SPH pair through the SPH pass, a single `dst[i] += src[j]` through the gather kernel,
// anything else as one kernel compiled from the bodies (pg_run_equations).  Bodies outside the
// equation grammar raise; there is no CPU fallback.
//
// Differences from the reference, all deliberate: equation() takes the body as text (C++ has
// no procedural macros); reads and writes keep first-appearance order (the reference collects
// them in HashSets, whose order is unspecified).
#pragma once

#include <cstddef>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/prestige_gpu.h"

namespace prestige {

struct EquationIR {
  std::string name;
  std::vector<std::string> reads;
  std::vector<std::string> writes;
  std::string body;
};

// Slice reads/writes of a pairwise body written in the reference's equation syntax, e.g.
// "force[i] += mass[j];".  Rules of prestige_macros/src/lib.rs:64-133: `x[..] = ...` and
// `x[..] op= ...` (the ten compound operators) write x; every `x[..]` reads x, including the
// left side of an assignment.  Field accesses (`a.x[i]`) are not slices.
EquationIR equation(const std::string& name, const std::string& body);

struct FusedEquations {
  std::vector<std::string> reads;
  std::vector<std::string> writes;
  std::vector<std::string> bodies;
};

FusedEquations fuse(const std::vector<EquationIR>& eqs);
std::string generate_simple_cpu(const FusedEquations& fused);
void debug_equation(const EquationIR& eq, std::ostream& os = std::cout);

// The fused SPH rates the CUDA pass evaluates together (continuity + momentum).
EquationIR sph_continuity();
EquationIR sph_momentum();

// Failure of a library call: its status (pg_status) and message.
class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

// One device-resident particle system (or a batch of independent SPH systems).
class System {
 public:
  System(const pg_config& cfg, size_t n);
  static System batch(const std::vector<pg_config>& cfgs, const std::vector<size_t>& counts);
  ~System();
  System(System&& o) noexcept;
  System& operator=(System&& o) noexcept;
  System(const System&) = delete;
  System& operator=(const System&) = delete;

  size_t size() const { return n_; }
  int dim() const { return dim_; }
  pg_system* raw() const { return h_; }

  // Named slices in particle-id order; vector slices interleaved (x0 y0 [z0] x1 ...).
  void set(const std::string& name, const std::vector<double>& values);
  std::vector<double> get(const std::string& name) const;

  // Asynchronous host I/O for step loops (f64 handles): set_async stages `values` (which must
  // stay valid and unchanged until wait_io) and the next call on the handle moves it into the
  // slice; get_async snapshots the slice now and fills `out` by wait_io.  Pinned host memory lets
  // the copies overlap the steps.
  void set_async(const std::string& name, const double* values, size_t count);
  void get_async(const std::string& name, double* out, size_t count);
  void wait_io();

  void step(int nsteps = 1);
  void step_async(int nsteps = 1);
  void compute_rates();
  void gather_sum(const std::string& dst, const std::string& src);
  void run_equations(const std::vector<std::string>& bodies);

  struct Gradients {
    double dL_dalpha = 0.0;
    double dL_dB = 0.0;
    std::vector<double> dL_dv0;
  };
  void forward_checkpointed(int nsteps, int every);
  Gradients backward(const std::vector<double>& dL_dx);

 private:
  System() = default;
  size_t components(const std::string& name) const;
  pg_system* h_ = nullptr;
  size_t n_ = 0;
  int dim_ = 3;
  int model_ = PG_MODEL_SPH;
};

// What run_gpu will do for a fused set, validated without touching a device.  Throws
// std::invalid_argument (with the translator's message) for a body outside the grammar.
struct GpuAction {
  enum Kind { GatherSum, SphRates, Compiled } kind;
  std::string dst, src;  // GatherSum: dst[i] += src[j]
};
std::vector<GpuAction> plan_gpu(const FusedEquations& fused);

// Executes a fused set on the GPU: the built-in SPH pair through pg_compute_rates; a single
// `dst[i] += src[j]` (the reference's eq1 form, prestige/src/lib.rs:10) through pg_gather_sum;
// any other set as one compiled kernel (pg_run_equations).
void run_gpu(const FusedEquations& fused, System& sys);

}  // namespace prestige
