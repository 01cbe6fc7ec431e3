// Implementation of prestige.hpp: the equation front end (text rules of the reference's
// #[equation] macro) and the C++ wrapper of the C ABI.
#include "prestige.hpp"

#include <algorithm>
#include <cctype>
#include <sstream>

namespace prestige {

namespace {

struct Token {
  enum Kind { Ident, Punct, Other } kind;
  std::string text;
};

// Identifiers, numbers and the punctuation of the equation syntax (longest match first).
std::vector<Token> tokenize(const std::string& s) {
  static const char* kOps[] = {"<<=", ">>=", "+=", "-=", "*=", "/=", "%=", "^=", "&=", "|=", "==", "!=",
                               "<=",  ">=",  "&&", "||", "<<", ">>", "->", "=>", "::", ".."};
  std::vector<Token> out;
  size_t i = 0;
  while (i < s.size()) {
    const unsigned char c = (unsigned char)s[i];
    if (std::isspace(c)) {
      ++i;
    } else if (std::isalpha(c) || c == '_') {
      size_t j = i + 1;
      while (j < s.size() && (std::isalnum((unsigned char)s[j]) || s[j] == '_')) ++j;
      out.push_back({Token::Ident, s.substr(i, j - i)});
      i = j;
    } else if (std::isdigit(c)) {
      size_t j = i + 1;
      while (j < s.size() && (std::isalnum((unsigned char)s[j]) || s[j] == '.' || s[j] == '_')) ++j;
      out.push_back({Token::Other, s.substr(i, j - i)});
      i = j;
    } else {
      std::string op(1, (char)c);
      for (const char* o : kOps) {
        const size_t L = std::char_traits<char>::length(o);
        if (s.compare(i, L, o) == 0) {
          op = o;
          break;
        }
      }
      out.push_back({Token::Punct, op});
      i += op.size();
    }
  }
  return out;
}

void add_unique(std::vector<std::string>& v, const std::string& s) {
  if (std::find(v.begin(), v.end(), s) == v.end()) v.push_back(s);
}

bool is_assign_op(const std::string& t) {
  static const char* kAssign[] = {"=", "+=", "-=", "*=", "/=", "%=", "^=", "&=", "|=", "<<=", ">>="};
  for (const char* a : kAssign)
    if (t == a) return true;
  return false;
}

// Index of the bracket closing the one opened at tokens[open].
size_t closing(const std::vector<Token>& t, size_t open) {
  int depth = 0;
  for (size_t k = open; k < t.size(); ++k) {
    if (t[k].kind != Token::Punct) continue;
    const std::string& p = t[k].text;
    if (p == "[" || p == "(" || p == "{") ++depth;
    if (p == "]" || p == ")" || p == "}") {
      if (--depth == 0) return k;
    }
  }
  return t.size();
}

// Body text without whitespace, enclosing braces or trailing semicolons.
std::string strip(const std::string& s) {
  std::string out;
  for (char c : s)
    if (!std::isspace((unsigned char)c)) out.push_back(c);
  while (out.size() >= 2 && out.front() == '{' && out.back() == '}') out = out.substr(1, out.size() - 2);
  while (!out.empty() && out.back() == ';') out.pop_back();
  return out;
}

}  // namespace

EquationIR equation(const std::string& name, const std::string& body) {
  EquationIR ir;
  ir.name = name;
  ir.body = body;
  const std::vector<Token> t = tokenize(body);
  // reads: every `x[` whose x is not a field (`a.x[`) -- in order of appearance
  for (size_t k = 0; k + 1 < t.size(); ++k) {
    if (t[k].kind == Token::Ident && t[k + 1].kind == Token::Punct && t[k + 1].text == "[" &&
        !(k > 0 && t[k - 1].kind == Token::Punct && t[k - 1].text == "."))
      add_unique(ir.reads, t[k].text);
  }
  // writes: statements `x[..] <assign-op> ...` at bracket depth 0
  size_t start = 0;
  for (size_t k = 0; k <= t.size(); ++k) {
    const bool end = k == t.size() ||
                     (t[k].kind == Token::Punct && (t[k].text == ";" || t[k].text == "{" || t[k].text == "}"));
    if (!end) continue;
    const size_t s0 = start;
    start = k + 1;
    if (k - s0 < 4) continue;  // shortest form: x [ i ] op ...
    if (t[s0].kind != Token::Ident || t[s0 + 1].text != "[") continue;
    if (s0 > 0 && t[s0 - 1].text == ".") continue;
    const size_t close = closing(t, s0 + 1);
    if (close + 1 < k && t[close + 1].kind == Token::Punct && is_assign_op(t[close + 1].text))
      add_unique(ir.writes, t[s0].text);
  }
  return ir;
}

FusedEquations fuse(const std::vector<EquationIR>& eqs) {
  FusedEquations f;
  for (const EquationIR& e : eqs) {
    for (const std::string& r : e.reads) add_unique(f.reads, r);
    for (const std::string& w : e.writes) add_unique(f.writes, w);
    f.bodies.push_back(e.body);
  }
  return f;
}

std::string generate_simple_cpu(const FusedEquations& fused) {
  std::string code = "for i in 0..n {\n    for j in 0..n {\n";
  for (const std::string& b : fused.bodies) code += "        " + b + "\n";
  code += "    }\n}\n";
  return code;
}

void debug_equation(const EquationIR& eq, std::ostream& os) {
  os << "----------------------\n";
  os << "Equation : " << eq.name << "\n";
  os << "Reads:\n";
  for (const std::string& r : eq.reads) os << "  " << r << "\n";
  os << "Writes:\n";
  for (const std::string& w : eq.writes) os << "  " << w << "\n";
  os << "Body:\n" << eq.body << "\n";
  os << "----------------------\n";
}

EquationIR sph_continuity() {
  return equation("sph_continuity", "drho[i] += mass[j] * dot(vel[i] - vel[j], grad_w(pos[i] - pos[j]));");
}

EquationIR sph_momentum() {
  return equation("sph_momentum",
                  "acc[i] -= mass[j] * (p[i] / (rho[i] * rho[i]) + p[j] / (rho[j] * rho[j]) + visc(i, j)) * "
                  "grad_w(pos[i] - pos[j]);");
}

// ---------------------------------------------------------------------------------------
// System
// ---------------------------------------------------------------------------------------
namespace {

void check(int status, const char* call) {
  if (status != PG_OK) throw Error(status, std::string(call) + ": " + pg_last_error());
}

}  // namespace

System::System(const pg_config& cfg, size_t n) {
  check(pg_create(&cfg, n, &h_), "pg_create");
  n_ = n;
  dim_ = cfg.dim;
  model_ = cfg.model;
}

System System::batch(const std::vector<pg_config>& cfgs, const std::vector<size_t>& counts) {
  if (cfgs.empty() || cfgs.size() != counts.size()) throw Error(PG_EINVAL, "batch: one count per configuration");
  System s;
  check(pg_batch_create(cfgs.data(), counts.data(), (int)cfgs.size(), &s.h_), "pg_batch_create");
  for (size_t c : counts) s.n_ += c;
  s.dim_ = cfgs[0].dim;
  s.model_ = cfgs[0].model;
  return s;
}

System::~System() {
  if (h_) pg_destroy(h_);
}

System::System(System&& o) noexcept : h_(o.h_), n_(o.n_), dim_(o.dim_), model_(o.model_) { o.h_ = nullptr; }

System& System::operator=(System&& o) noexcept {
  if (this != &o) {
    if (h_) pg_destroy(h_);
    h_ = o.h_;
    n_ = o.n_;
    dim_ = o.dim_;
    model_ = o.model_;
    o.h_ = nullptr;
  }
  return *this;
}

size_t System::components(const std::string& name) const {
  if (name == "pos" || name == "vel" || name == "acc") return model_ == PG_MODEL_DEM ? 3 : (size_t)dim_;
  if (name == "omega") return 3;
  return 1;
}

void System::set(const std::string& name, const std::vector<double>& values) {
  check(pg_set_field(h_, name.c_str(), values.data(), values.size(), PG_F64), "pg_set_field");
}

std::vector<double> System::get(const std::string& name) const {
  std::vector<double> out(n_ * components(name));
  check(pg_get_field(h_, name.c_str(), out.data(), out.size(), PG_F64), "pg_get_field");
  return out;
}

void System::set_async(const std::string& name, const double* values, size_t count) {
  check(pg_set_field_async(h_, name.c_str(), values, count, PG_F64), "pg_set_field_async");
}

void System::get_async(const std::string& name, double* out, size_t count) {
  check(pg_get_field_async(h_, name.c_str(), out, count, PG_F64), "pg_get_field_async");
}

void System::wait_io() { check(pg_wait_io(h_), "pg_wait_io"); }

void System::step(int nsteps) { check(pg_step(h_, nsteps), "pg_step"); }

void System::step_async(int nsteps) { check(pg_step_async(h_, nsteps), "pg_step_async"); }

void System::compute_rates() { check(pg_compute_rates(h_), "pg_compute_rates"); }

void System::gather_sum(const std::string& dst, const std::string& src) {
  check(pg_gather_sum(h_, dst.c_str(), src.c_str()), "pg_gather_sum");
}

void System::run_equations(const std::vector<std::string>& bodies) {
  std::vector<const char*> b;
  for (const std::string& x : bodies) b.push_back(x.c_str());
  check(pg_run_equations(h_, b.data(), (int)b.size()), "pg_run_equations");
}

void System::forward_checkpointed(int nsteps, int every) {
  check(pg_forward_checkpointed(h_, nsteps, every), "pg_forward_checkpointed");
}

System::Gradients System::backward(const std::vector<double>& dL_dx) {
  if (dL_dx.size() != n_ * (size_t)dim_) throw Error(PG_EINVAL, "backward: dL/dx needs n * dim values");
  Gradients g;
  g.dL_dv0.resize(n_ * (size_t)dim_);
  check(pg_backward(h_, dL_dx.data(), &g.dL_dalpha, &g.dL_dB, g.dL_dv0.data()), "pg_backward");
  return g;
}

// ---------------------------------------------------------------------------------------
// GPU backend
// ---------------------------------------------------------------------------------------
std::vector<GpuAction> plan_gpu(const FusedEquations& fused) {
  if (fused.bodies.empty()) throw std::invalid_argument("empty equation set");
  const std::string cont = strip(sph_continuity().body), mom = strip(sph_momentum().body);
  bool all_sph = true;
  for (const std::string& b : fused.bodies) {
    const std::string s = strip(b);
    all_sph = all_sph && (s == cont || s == mom);
  }
  if (all_sph) return {GpuAction{GpuAction::SphRates, "", ""}};
  if (fused.bodies.size() == 1) {  // exactly `dst[i] += src[j]`
    const std::vector<Token> t = tokenize(fused.bodies[0]);
    size_t m = t.size();
    while (m > 0 && t[m - 1].text == ";") --m;
    const bool ok = m == 9 && t[0].kind == Token::Ident && t[1].text == "[" && t[2].text == "i" && t[3].text == "]" &&
                    t[4].text == "+=" && t[5].kind == Token::Ident && t[6].text == "[" && t[7].text == "j" &&
                    t[8].text == "]";
    if (ok) return {GpuAction{GpuAction::GatherSum, t[0].text, t[5].text}};
  }
  // anything else: one compiled kernel; validate with the library's translator
  std::vector<const char*> b;
  for (const std::string& x : fused.bodies) b.push_back(x.c_str());
  size_t need = 0;
  if (pg_equation_source(b.data(), (int)b.size(), nullptr, 0, &need) != PG_OK)
    throw std::invalid_argument(std::string("equation set refused: ") + pg_last_error());
  return {GpuAction{GpuAction::Compiled, "", ""}};
}

void run_gpu(const FusedEquations& fused, System& sys) {
  for (const GpuAction& a : plan_gpu(fused)) {
    if (a.kind == GpuAction::SphRates) sys.compute_rates();
    else if (a.kind == GpuAction::GatherSum) sys.gather_sum(a.dst, a.src);
    else sys.run_equations(fused.bodies);
  }
}

}  // namespace prestige
