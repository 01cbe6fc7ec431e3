// GPU execution of pairwise equations given as source text.
//
// The reference turns fused equations into the text of a CPU loop
// (prestige/src/codegen/simple_cpu.rs:3-22: `for i in 0..n { for j in 0..n { bodies } }`) and
// never runs it.  This file turns the same bodies into a CUDA gather over the cell list --
// for each particle i, the bodies run for every neighbour j with |x_i - x_j| < support
// (j == i included), in the traversal order of pg_gather_sum -- compiles it at run time with
// NVRTC for the device, and launches it on the handle's stream.
//
// Body syntax (the subset of Rust expressions an #[equation] body uses):
//   statements      `x[i] = e`, `x[i] += e` (also -=, *=, /=), `let name = e` (`let name: f64 = e`),
//                   separated by `;`; a body may be wrapped in braces
//   expressions     numbers, + - * / and parentheses, slices `x[i]` / `x[j]`, let-bound names,
//                   the pair geometry `dx dy dz` (x_i - x_j), `r2`, `r`, the support `support`,
//                   functions sqrt exp ln abs min max powi powf sin cos, called as f(a, ..) or
//                   as Rust methods a.f(..)
// Slices are double fields of the handle: user fields (pg_set_field) and, in double-precision
// systems, the built-in scalars "mass" and "rho" (read-only).  Only `x[i]` may be assigned.
// Semantics: every statement of every body runs in order for each (i, j); reads of x[i] see
// the value accumulated so far for i; reads of x[j] see the values before the call (the
// reference's sequential loop would see already-updated x[j] for j < i, an order dependence a
// parallel gather cannot keep).  All arithmetic is IEEE double without contraction, so
// `force[i] += mass[j]` reproduces pg_gather_sum bit for bit.
//
// NVRTC is loaded with dlopen on first use, so the library still loads where it is absent.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cctype>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "pg_internal.cuh"
#include "pg_kernels.cuh"
#include "pg_system.cuh"

namespace pg {
namespace {

// ---------------------------------------------------------------------------------------
// Tokens
// ---------------------------------------------------------------------------------------
struct Tok {
  enum Kind { Ident, Num, Punct } kind;
  std::string s;
};

bool tokenize(const std::string& src, std::vector<Tok>& out, std::string& err) {
  static const char* kOps[] = {"+=", "-=", "*=", "/=", "==", "!=", "<=", ">=", "&&", "||", "::", "->"};
  size_t i = 0;
  while (i < src.size()) {
    const unsigned char c = (unsigned char)src[i];
    if (std::isspace(c)) {
      ++i;
    } else if (std::isalpha(c) || c == '_') {
      size_t j = i + 1;
      while (j < src.size() && (std::isalnum((unsigned char)src[j]) || src[j] == '_')) ++j;
      out.push_back({Tok::Ident, src.substr(i, j - i)});
      i = j;
    } else if (std::isdigit(c) || (c == '.' && i + 1 < src.size() && std::isdigit((unsigned char)src[i + 1]))) {
      size_t j = i;
      bool dot = false, exp = false;
      while (j < src.size()) {
        const char d = src[j];
        if (std::isdigit((unsigned char)d) || d == '_') {
          ++j;
        } else if (d == '.' && !dot && !exp && !(j + 1 < src.size() && std::isalpha((unsigned char)src[j + 1]))) {
          dot = true;
          ++j;
        } else if ((d == 'e' || d == 'E') && !exp) {
          exp = true;
          ++j;
          if (j < src.size() && (src[j] == '+' || src[j] == '-')) ++j;
        } else {
          break;
        }
      }
      std::string num;
      for (size_t k = i; k < j; ++k)
        if (src[k] != '_') num.push_back(src[k]);
      if (j + 3 <= src.size() && src.compare(j, 3, "f64") == 0) j += 3;  // 1.0f64
      if (!dot && !exp) num += ".0";  // integer literals are doubles in equation arithmetic
      out.push_back({Tok::Num, num});
      i = j;
    } else {
      std::string op(1, (char)c);
      for (const char* o : kOps)
        if (src.compare(i, strlen(o), o) == 0) {
          op = o;
          break;
        }
      if (std::string("+-*/()[]{};,.:=").find(op[0]) == std::string::npos || op == "==" || op == "!=" ||
          op == "<=" || op == ">=" || op == "&&" || op == "||" || op == "::" || op == "->") {
        err = "unsupported token '" + op + "'";
        return false;
      }
      out.push_back({Tok::Punct, op});
      i += op.size();
    }
  }
  return true;
}

// ---------------------------------------------------------------------------------------
// Translation of one fused set into the body of the generated kernel.
// ---------------------------------------------------------------------------------------
struct Slice {
  bool read_i = false, read_j = false, written = false;
};

struct Translation {
  std::map<std::string, Slice> slices;  // by name
  std::set<std::string> geometry;       // dx dy dz r2 r used
  std::string code;                     // the statements, one brace block per body
};

const std::map<std::string, std::string>& functions() {
  static const std::map<std::string, std::string> f = {
      {"sqrt", "sqrt"}, {"exp", "exp"},   {"ln", "log"},   {"abs", "fabs"},  {"min", "fmin"},
      {"max", "fmax"},  {"powi", "pg_powi"}, {"powf", "pow"}, {"sin", "sin"}, {"cos", "cos"}};
  return f;
}

bool is_geometry(const std::string& s) {
  return s == "dx" || s == "dy" || s == "dz" || s == "r2" || s == "r" || s == "support";
}

std::string slice_var(const std::string& name, char side) { return "pg_" + name + "_" + side; }

// Expression tokens [b, e) -> C++ text.
bool expr(const std::vector<Tok>& t, size_t b, size_t e, const std::set<std::string>& locals, Translation& tr,
          std::string& out, std::string& err) {
  std::vector<std::string> o;           // output pieces
  std::vector<size_t> open;             // output index where each open group starts
  size_t last_start = std::string::npos;  // output index where the last complete operand starts
  for (size_t k = b; k < e; ++k) {
    const Tok& x = t[k];
    if (x.kind == Tok::Num) {
      last_start = o.size();
      o.push_back(x.s);
    } else if (x.kind == Tok::Ident) {
      if (k + 1 < e && t[k + 1].s == "[") {  // slice
        if (k + 3 >= e || t[k + 3].s != "]" || (t[k + 2].s != "i" && t[k + 2].s != "j")) {
          err = "slice '" + x.s + "' must be indexed by i or j";
          return false;
        }
        const char side = t[k + 2].s[0];
        Slice& sl = tr.slices[x.s];
        (side == 'i' ? sl.read_i : sl.read_j) = true;
        last_start = o.size();
        o.push_back(slice_var(x.s, side));
        k += 3;
      } else if (k + 1 < e && t[k + 1].s == "(") {  // function call
        auto f = functions().find(x.s);
        if (f == functions().end()) {
          err = "unknown function '" + x.s + "'";
          return false;
        }
        open.push_back(o.size());
        o.push_back(f->second + "(");
        ++k;
      } else if (locals.count(x.s)) {
        last_start = o.size();
        o.push_back(x.s);
      } else if (is_geometry(x.s)) {
        if (x.s != "support") tr.geometry.insert(x.s);
        last_start = o.size();
        o.push_back(x.s == "support" ? "pg_support" : "pg_" + x.s);
      } else {
        err = "unknown name '" + x.s + "'";
        return false;
      }
    } else if (x.s == "(") {
      open.push_back(o.size());
      o.push_back("(");
    } else if (x.s == ")") {
      if (open.empty()) {
        err = "unbalanced ')'";
        return false;
      }
      last_start = open.back();
      open.pop_back();
      o.push_back(")");
    } else if (x.s == ".") {  // method call on the last operand: a.f(args) -> f(a, args)
      if (last_start == std::string::npos || k + 2 >= e || t[k + 1].kind != Tok::Ident || t[k + 2].s != "(") {
        err = "'.' must be a method call on an operand";
        return false;
      }
      auto f = functions().find(t[k + 1].s);
      if (f == functions().end()) {
        err = "unknown method '" + t[k + 1].s + "'";
        return false;
      }
      std::string operand;
      for (size_t q = last_start; q < o.size(); ++q) operand += o[q];
      o.resize(last_start);
      const bool no_args = k + 3 < e && t[k + 3].s == ")";
      open.push_back(o.size());
      o.push_back(f->second + "(" + operand + (no_args ? "" : ", "));
      k += 2;
    } else if (x.s == "+" || x.s == "-" || x.s == "*" || x.s == "/" || x.s == ",") {
      o.push_back(" " + x.s + " ");
      last_start = std::string::npos;
    } else {
      err = "unexpected '" + x.s + "' in an expression";
      return false;
    }
  }
  if (!open.empty()) {
    err = "unbalanced '('";
    return false;
  }
  out.clear();
  for (const std::string& p : o) out += p;
  if (out.empty()) {
    err = "empty expression";
    return false;
  }
  return true;
}

bool translate(const std::vector<std::string>& bodies, Translation& tr, std::string& err) {
  for (size_t bi = 0; bi < bodies.size(); ++bi) {
    std::vector<Tok> t;
    if (!tokenize(bodies[bi], t, err)) return false;
    while (!t.empty() && t.front().s == "{" && t.back().s == "}") t = std::vector<Tok>(t.begin() + 1, t.end() - 1);
    std::set<std::string> locals;
    tr.code += "    {\n";
    size_t s0 = 0;
    for (size_t k = 0; k <= t.size(); ++k) {
      if (k < t.size() && t[k].s != ";") continue;
      const size_t a = s0, b = k;
      s0 = k + 1;
      if (a == b) continue;
      std::string rhs;
      if (t[a].s == "let") {
        if (b - a < 4 || t[a + 1].kind != Tok::Ident) {
          err = "malformed let";
          return false;
        }
        size_t eq = a + 2;
        if (t[eq].s == ":") eq += 2;  // let name: f64 = ...
        if (eq >= b || t[eq].s != "=") {
          err = "malformed let";
          return false;
        }
        const std::string& name = t[a + 1].s;
        if (name.compare(0, 3, "pg_") == 0 || functions().count(name) || is_geometry(name)) {
          err = "reserved name '" + name + "'";
          return false;
        }
        if (!expr(t, eq + 1, b, locals, tr, rhs, err)) return false;
        locals.insert(name);
        tr.code += "      const double " + name + " = " + rhs + ";\n";
        continue;
      }
      // x[i] op= rhs
      if (b - a < 6 || t[a].kind != Tok::Ident || t[a + 1].s != "[" || t[a + 3].s != "]") {
        err = "a statement must be `let name = e` or `x[i] op= e`";
        return false;
      }
      if (t[a + 2].s != "i") {
        err = "only x[i] may be assigned (got '" + t[a].s + "[" + t[a + 2].s + "]'); a gather cannot write x[j]";
        return false;
      }
      const std::string op = t[a + 4].s;
      if (op != "=" && op != "+=" && op != "-=" && op != "*=" && op != "/=") {
        err = "unsupported assignment '" + op + "'";
        return false;
      }
      if (!expr(t, a + 5, b, locals, tr, rhs, err)) return false;
      Slice& sl = tr.slices[t[a].s];
      sl.written = true;
      sl.read_i = true;  // the accumulator starts from the stored value
      tr.code += "      " + slice_var(t[a].s, 'i') + " " + op + " " + rhs + ";\n";
    }
    tr.code += "    }\n";
  }
  return true;
}

// Kernel source for a translation.  P: "double" or "float" (the system precision).
std::string kernel_source(const Translation& tr, const char* P, const std::vector<std::string>& order,
                          const std::vector<std::string>& types) {
  std::string src;
  src += "typedef " + std::string(P) + " P;\n";
  src += std::string("struct __align__(") + (strcmp(P, "double") == 0 ? "32" : "16") + ") P4 { P x, y, z, w; };\n";
  src += "struct PgEqGrid { double support; P support2; int nx, ny, nz, reach, dim; unsigned n; };\n";
  src += "__device__ __forceinline__ double pg_powi(double x, double e) {\n"
         "  int n = (int)e; double r = 1.0, b = n < 0 ? 1.0 / x : x; n = n < 0 ? -n : n;\n"
         "  for (; n; n >>= 1) { if (n & 1) r *= b; b *= b; } return r; }\n";
  src += "extern \"C\" __global__ void pg_equations(PgEqGrid G, const P4* __restrict__ spos,\n"
         "    const unsigned* __restrict__ sorted_id, const unsigned* __restrict__ sorted_cell,\n"
         "    const unsigned* __restrict__ cell_start";
  // per slice: pg_p_ (the i side, written in place) and pg_q_ (the j side: the same buffer, or a
  // snapshot taken before the launch when the slice is also written)
  for (size_t f = 0; f < order.size(); ++f) {
    const bool w = tr.slices.at(order[f]).written;
    src += ", " + std::string(w ? "" : "const ") + types[f] + "* " + (w ? "" : "__restrict__ ") + "pg_p_" + order[f];
    src += ", const " + types[f] + "* pg_q_" + order[f];
  }
  src += ") {\n";
  src += "  const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;\n  if (k >= G.n) return;\n";
  src += "  const unsigned id = sorted_id[k];\n  const P4 pi = spos[k];\n  const double pg_support = G.support;\n";
  for (const std::string& name : order) {
    const Slice& sl = tr.slices.at(name);
    if (sl.read_i || sl.written)
      src += "  double " + slice_var(name, 'i') + " = (double)pg_p_" + name + "[id];\n";
  }
  src += "  const unsigned c = sorted_cell[k];\n"
         "  const int cx = (int)(c % (unsigned)G.nx), cy = (int)((c / (unsigned)G.nx) % (unsigned)G.ny);\n"
         "  const int cz = (int)(c / ((unsigned)G.nx * (unsigned)G.ny));\n"
         "  const int R = G.reach, RZ = G.dim == 3 ? R : 0;\n"
         "  const int x0 = max(cx - R, 0), x1 = min(cx + R, G.nx - 1);\n"
         "  for (int dzc = -RZ; dzc <= RZ; ++dzc) {\n    const int zc = cz + dzc;\n"
         "    if (zc < 0 || zc >= G.nz) continue;\n"
         "    for (int dyc = -R; dyc <= R; ++dyc) {\n      const int yc = cy + dyc;\n"
         "      if (yc < 0 || yc >= G.ny) continue;\n"
         "      const unsigned rb = ((unsigned)zc * G.ny + (unsigned)yc) * G.nx;\n"
         "      const unsigned s = cell_start[rb + x0], e = cell_start[rb + x1 + 1];\n"
         "      for (unsigned t = s; t < e; ++t) {\n"
         "        const P4 pj = spos[t];\n"
         "        const P d0 = pi.x - pj.x, d1 = pi.y - pj.y, d2 = G.dim == 3 ? pi.z - pj.z : (P)0;\n"
         "        P rr = d0 * d0 + d1 * d1;\n        if (G.dim == 3) rr = rr + d2 * d2;\n"
         "        if (!(rr < G.support2)) continue;\n"
         "        const unsigned j = sorted_id[t];\n        (void)j;\n";
  if (tr.geometry.count("dx")) src += "        const double pg_dx = (double)d0;\n";
  if (tr.geometry.count("dy")) src += "        const double pg_dy = (double)d1;\n";
  if (tr.geometry.count("dz")) src += "        const double pg_dz = (double)d2;\n";
  if (tr.geometry.count("r2") || tr.geometry.count("r")) src += "        const double pg_r2 = (double)rr;\n";
  if (tr.geometry.count("r")) src += "        const double pg_r = sqrt(pg_r2);\n";
  for (const std::string& name : order)
    if (tr.slices.at(name).read_j)
      src += "        const double " + slice_var(name, 'j') + " = (double)pg_q_" + name + "[j];\n";
  // statement blocks, indented into the loop
  std::string code = tr.code;
  std::string ind;
  for (size_t p = 0; p < code.size(); ++p) {
    if (p == 0 || code[p - 1] == '\n') ind += "      ";
    ind += code[p];
  }
  src += ind;
  src += "      }\n    }\n  }\n";
  for (const std::string& name : order)
    if (tr.slices.at(name).written) src += "  pg_p_" + name + "[id] = " + slice_var(name, 'i') + ";\n";
  src += "}\n";
  return src;
}

// ---------------------------------------------------------------------------------------
// NVRTC (dlopen) and the compiled-kernel cache
// ---------------------------------------------------------------------------------------
struct Nvrtc {
  bool tried = false, ok = false;
  std::string why;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcGetErrorString) error_string = nullptr;
};

std::mutex g_jit_mu;
Nvrtc g_nvrtc;
std::map<std::string, cudaKernel_t> g_kernels;  // key: device + source

bool load_nvrtc(std::string& err) {
  Nvrtc& n = g_nvrtc;
  if (n.tried) {
    err = n.why;
    return n.ok;
  }
  n.tried = true;
  void* h = nullptr;
  for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"})
    if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
  if (!h) {
    n.why = "NVRTC (libnvrtc.so) is not available: run-time equation kernels cannot be compiled";
    err = n.why;
    return false;
  }
#define PG_SYM(field, sym) n.field = (decltype(n.field))dlsym(h, #sym)
  PG_SYM(create, nvrtcCreateProgram);
  PG_SYM(compile, nvrtcCompileProgram);
  PG_SYM(log_size, nvrtcGetProgramLogSize);
  PG_SYM(log, nvrtcGetProgramLog);
  PG_SYM(cubin_size, nvrtcGetCUBINSize);
  PG_SYM(cubin, nvrtcGetCUBIN);
  PG_SYM(destroy, nvrtcDestroyProgram);
  PG_SYM(error_string, nvrtcGetErrorString);
#undef PG_SYM
  n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy && n.error_string;
  if (!n.ok) n.why = "libnvrtc.so lacks an expected entry point";
  err = n.why;
  return n.ok;
}

int compile_kernel(const std::string& src, cudaKernel_t* out) {
  int dev = 0, major = 0, minor = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev));
  PG_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  PG_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  const std::string key = std::to_string(dev) + "\n" + src;
  std::lock_guard<std::mutex> lock(g_jit_mu);
  auto it = g_kernels.find(key);
  if (it != g_kernels.end()) {
    *out = it->second;
    return PG_OK;
  }
  std::string err;
  if (!load_nvrtc(err)) {
    set_error("%s", err.c_str());
    return PG_ESTATE;
  }
  Nvrtc& n = g_nvrtc;
  nvrtcProgram prog;
  if (n.create(&prog, src.c_str(), "pg_equations.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
    set_error("nvrtcCreateProgram failed");
    return PG_ECUDA;
  }
  char arch[64];
  snprintf(arch, sizeof(arch), "--gpu-architecture=sm_%d%d", major, minor);
  const char* opts[] = {arch, "--fmad=false", "--std=c++17"};
  const nvrtcResult cr = n.compile(prog, 3, opts);
  if (cr != NVRTC_SUCCESS) {
    size_t ls = 0;
    n.log_size(prog, &ls);
    std::string log(ls, '\0');
    if (ls) n.log(prog, &log[0]);
    n.destroy(&prog);
    set_error("equation kernel did not compile: %s\n%s", n.error_string(cr), log.c_str());
    return PG_EINVAL;
  }
  size_t cs = 0;
  n.cubin_size(prog, &cs);
  std::vector<char> cubin(cs);
  n.cubin(prog, cubin.data());
  n.destroy(&prog);
  cudaLibrary_t lib;
  PG_CUDA_TRY(cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  cudaKernel_t kern;
  PG_CUDA_TRY(cudaLibraryGetKernel(&kern, lib, "pg_equations"));
  g_kernels[key] = kern;  // the library stays loaded for the life of the process
  *out = kern;
  return PG_OK;
}

bool to_bodies(const char* const* bodies, int n_bodies, std::vector<std::string>& v) {
  if (!bodies || n_bodies < 1) return false;
  for (int b = 0; b < n_bodies; ++b) {
    if (!bodies[b]) return false;
    v.emplace_back(bodies[b]);
  }
  return true;
}

}  // namespace
}  // namespace pg

extern "C" {

int pg_equation_source(const char* const* bodies, int n_bodies, char* out, size_t capacity, size_t* needed) {
  pg::clear_error();
  std::vector<std::string> v;
  if (!pg::to_bodies(bodies, n_bodies, v)) {
    pg::set_error("need n_bodies >= 1 non-null bodies");
    return PG_EINVAL;
  }
  pg::Translation tr;
  std::string err;
  if (!pg::translate(v, tr, err)) {
    pg::set_error("equation: %s", err.c_str());
    return PG_EINVAL;
  }
  std::vector<std::string> order, types;
  for (const auto& kv : tr.slices) {
    order.push_back(kv.first);
    types.push_back("double");
  }
  const std::string src = pg::kernel_source(tr, "double", order, types);
  if (needed) *needed = src.size() + 1;
  if (out && capacity) {
    const size_t m = std::min(capacity - 1, src.size());
    memcpy(out, src.data(), m);
    out[m] = 0;
    if (m < src.size()) {
      pg::set_error("output buffer too small (%zu bytes needed)", src.size() + 1);
      return PG_EOVERFLOW;
    }
  }
  return PG_OK;
}

int pg_run_equations(pg_system* s, const char* const* bodies, int n_bodies) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  std::vector<std::string> v;
  if (!pg::to_bodies(bodies, n_bodies, v)) {
    pg::set_error("need n_bodies >= 1 non-null bodies");
    return PG_EINVAL;
  }
  if (s->nsys != 1) {
    pg::set_error("pg_run_equations runs on single-system handles");
    return PG_EINVAL;
  }
  pg::Translation tr;
  std::string err;
  if (!pg::translate(v, tr, err)) {
    pg::set_error("equation: %s", err.c_str());
    return PG_EINVAL;
  }
  // bind slices to device buffers; a slice written at i and read at j is read from a snapshot
  std::vector<std::string> order, types;
  std::vector<void*> ptrs, jptrs;
  for (const auto& kv : tr.slices) {
    const std::string& name = kv.first;
    const bool builtin = (name == "mass" || name == "rho") && s->model == PG_MODEL_SPH;
    pg::DevBuf* buf = nullptr;
    std::string type = "double";
    if (builtin) {
      if (kv.second.written) {
        pg::set_error("slice '%s' is read-only in equations", name.c_str());
        return PG_EINVAL;
      }
      buf = name == "mass" ? &s->mass : &s->rho;
      if (!s->f64) type = "float";
    } else {
      auto it = s->user.find(name);
      if (it == s->user.end()) {
        pg::set_error("unknown slice '%s' (create it with pg_set_field)", name.c_str());
        return PG_ENOTFOUND;
      }
      buf = it->second.get();
    }
    order.push_back(name);
    types.push_back(type);
    ptrs.push_back(buf->p);
    void* jp = buf->p;
    if (kv.second.written && kv.second.read_j) {
      std::unique_ptr<pg::DevBuf>& snap = s->snapshots[name];
      if (!snap) snap.reset(new pg::DevBuf());
      PG_TRY(snap->ensure(8 * (s->n ? s->n : 1)));
      if (s->n) PG_CUDA_TRY(cudaMemcpyAsync(snap->p, buf->p, 8 * s->n, cudaMemcpyDeviceToDevice, s->stream));
      jp = snap->p;
    }
    jptrs.push_back(jp);
  }
  const std::string src = pg::kernel_source(tr, s->f64 ? "double" : "float", order, types);
  cudaKernel_t kern;
  PG_TRY(pg::compile_kernel(src, &kern));
  PG_TRY(pg_build_neighbors(s));
  // kernel arguments: grid record, sorted positions, sorted ids and cells, cell table, slices
  struct GridD {
    double support;
    double support2;
    int nx, ny, nz, reach, dim;
    unsigned n;
  } gd;
  struct GridF {
    double support;
    float support2;
    int nx, ny, nz, reach, dim;
    unsigned n;
  } gf;
  const pg::Grid& g = s->grids[0];
  void* grid_arg;
  if (s->f64) {
    gd = {g.support, g.support * g.support, g.n[0], g.n[1], g.n[2], g.reach, s->dim, (unsigned)s->n};
    grid_arg = &gd;
  } else {
    const float sf = (float)g.support;
    gf = {g.support, sf * sf, g.n[0], g.n[1], g.n[2], g.reach, s->dim, (unsigned)s->n};
    grid_arg = &gf;
  }
  const void* spos = s->spos.p;
  const void* sid = s->nw.sorted_id;
  const void* scell = s->nw.sorted_cell;
  const void* cstart = s->nw.cell_start.p;
  std::vector<void*> args = {grid_arg, (void*)&spos, (void*)&sid, (void*)&scell, (void*)&cstart};
  for (size_t f = 0; f < ptrs.size(); ++f) {
    args.push_back(&ptrs[f]);
    args.push_back(&jptrs[f]);
  }
  if (s->n) {
    const unsigned blocks = (unsigned)((s->n + 127) / 128);
    PG_CUDA_TRY(cudaLaunchKernel((const void*)kern, dim3(blocks), dim3(128), args.data(), 0, s->stream));
  }
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

}  // extern "C"
