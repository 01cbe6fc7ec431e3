// Tests of the C++ host layer (prestige_gb300/host/prestige.hpp), run by tests/test_cpp_host.py.
//
//   test_host cpu   the equation front end: the reference's two tests (prestige/src/lib.rs:20-52,
//                   which only print) restated with assertions, plus the SliceVisitor rules of
//                   prestige_macros/src/lib.rs:64-133 and the GPU plan (no device needed)
//   test_host gpu   eq1 (force[i] += mass[j], prestige/src/lib.rs:7-12) run through run_gpu on a
//                   System against brute force over all pairs, bit for bit; an SPH step and a
//                   checkpointed adjoint through the C++ API
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../prestige_gb300/host/prestige.hpp"

static int g_failures = 0;
#define CHECK(cond)                                                          \
  do {                                                                       \
    if (!(cond)) {                                                           \
      std::fprintf(stderr, "%s:%d: CHECK failed: %s\n", __FILE__, __LINE__, #cond); \
      ++g_failures;                                                          \
    }                                                                        \
  } while (0)

using namespace prestige;

static std::set<std::string> as_set(const std::vector<std::string>& v) { return std::set<std::string>(v.begin(), v.end()); }

// prestige/src/lib.rs:7-12
static EquationIR eq1() { return equation("eq1", "force[i] += mass[j];"); }

static void test_equation_ir() {
  const EquationIR ir = eq1();
  CHECK(ir.name == "eq1");
  CHECK(as_set(ir.reads) == (std::set<std::string>{"force", "mass"}));
  CHECK(ir.writes == std::vector<std::string>{"force"});
  std::ostringstream os;
  debug_equation(ir, os);
  const std::string out = os.str();
  CHECK(out.find("Equation : eq1") != std::string::npos);
  CHECK(out.find("Reads:\n") != std::string::npos && out.find("  force\n") != std::string::npos);
  CHECK(out.find("Writes:\n  force\n") != std::string::npos);
}

static void test_fusion() {
  const FusedEquations f = fuse({eq1()});
  CHECK(as_set(f.reads) == (std::set<std::string>{"force", "mass"}));
  CHECK(as_set(f.writes) == (std::set<std::string>{"force"}));
  CHECK(generate_simple_cpu(f) ==
        "for i in 0..n {\n    for j in 0..n {\n        force[i] += mass[j];\n    }\n}\n");
}

static void test_slice_rules() {
  const char* ops[] = {"+=", "-=", "*=", "/=", "%=", "^=", "&=", "|=", "<<=", ">>="};
  for (const char* op : ops) {
    const EquationIR ir = equation("c", std::string("x[i] ") + op + " y[j];");
    CHECK(ir.writes == std::vector<std::string>{"x"});
    CHECK(as_set(ir.reads) == (std::set<std::string>{"x", "y"}));
  }
  EquationIR a = equation("a", "a[i] = b[j] * c[i] + 2.0;");
  CHECK(a.writes == std::vector<std::string>{"a"});
  CHECK(as_set(a.reads) == (std::set<std::string>{"a", "b", "c"}));
  EquationIR l = equation("l", "let t = p[j] * 0.5; q[i] += t; s.f[i] = 1.0;");
  CHECK(l.writes == std::vector<std::string>{"q"});
  CHECK(as_set(l.reads) == (std::set<std::string>{"p", "q"}));
  EquationIR cmp = equation("cmp", "if u[i] == v[j] { w[i] += 1.0; }");
  CHECK(cmp.writes == std::vector<std::string>{"w"});
  const FusedEquations two = fuse({eq1(), equation("eq2", "acc[i] -= mass[j] * vel[j];")});
  CHECK(as_set(two.reads) == (std::set<std::string>{"force", "mass", "acc", "vel"}));
  CHECK(two.bodies.size() == 2 && two.bodies[1] == "acc[i] -= mass[j] * vel[j];");
}

static void test_gpu_plan() {
  const std::vector<GpuAction> p = plan_gpu(fuse({eq1()}));
  CHECK(p.size() == 1 && p[0].kind == GpuAction::GatherSum && p[0].dst == "force" && p[0].src == "mass");
  const std::vector<GpuAction> q = plan_gpu(fuse({sph_continuity(), sph_momentum()}));
  CHECK(q.size() == 1 && q[0].kind == GpuAction::SphRates);
  const std::vector<GpuAction> c = plan_gpu(fuse({eq1(), equation("odd", "a[i] *= b[j] * r;")}));
  CHECK(c.size() == 1 && c[0].kind == GpuAction::Compiled);
  bool threw = false;
  try {
    plan_gpu(fuse({equation("bad", "a[j] += b[i];")}));  // a gather cannot write x[j]
  } catch (const std::invalid_argument& e) {
    threw = std::string(e.what()).find("only x[i] may be assigned") != std::string::npos;
  }
  CHECK(threw);
}

// ---------------------------------------------------------------------------------------
static pg_config sph_config(int dim, double h, double lo, double hi) {
  pg_config c;
  pg_config_default(&c);
  c.dim = dim;
  c.h = h;
  for (int d = 0; d < 3; ++d) {
    c.domain_lo[d] = d < dim ? lo : 0.0;
    c.domain_hi[d] = d < dim ? hi : 0.0;
  }
  c.tait_B = 1000.0 * 100.0 / 7.0;
  return c;
}

static void test_gpu_eq1_bit_exact() {
  const int n = 3000, dim = 3;
  const double h = 0.01, support = 2 * h;
  std::mt19937_64 rng(5);
  std::uniform_real_distribution<double> U(0.0, 0.2);
  std::uniform_int_distribution<int> M(1, 1000);
  std::vector<double> pos(n * dim), mass(n), force(n, 0.0);
  for (auto& p : pos) p = U(rng);
  for (auto& m : mass) m = M(rng);
  System sys(sph_config(dim, h, 0.0, 0.2), n);
  sys.set("pos", pos);
  sys.set("mass", mass);
  sys.set("force", force);
  run_gpu(fuse({eq1()}), sys);
  const std::vector<double> got = sys.get("force");
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    double ref = 0.0;
    for (int j = 0; j < n; ++j) {
      const double d0 = pos[3 * i] - pos[3 * j], d1 = pos[3 * i + 1] - pos[3 * j + 1], d2 = pos[3 * i + 2] - pos[3 * j + 2];
      const double r2 = (d0 * d0 + d1 * d1) + d2 * d2;
      if (r2 < support * support) ref += mass[j];
    }
    if (got[i] != ref) ++bad;
  }
  CHECK(bad == 0);
}

static void test_gpu_compiled_equations() {
  const int n = 2000, dim = 3;
  std::mt19937_64 rng(9);
  std::uniform_real_distribution<double> U(0.0, 0.2);
  std::vector<double> pos(n * dim), mass(n, 1.0), a(n, 1.0), c(n, 0.0);
  for (auto& p : pos) p = U(rng);
  System sys(sph_config(dim, 0.01, 0.0, 0.2), n);
  sys.set("pos", pos);
  sys.set("m2", mass);
  sys.set("a", a);
  sys.set("c", c);
  // two fused bodies: reads of a[j] see the values before the call
  run_gpu(fuse({equation("e1", "a[i] += m2[j];"), equation("e2", "c[i] += a[j] * 2.0;")}), sys);
  const std::vector<double> ga = sys.get("a"), gc = sys.get("c");
  int bad = 0;
  for (int i = 0; i < n; ++i)
    if (gc[i] != 2.0 * (ga[i] - 1.0)) ++bad;  // every neighbour has m2 = a = 1
  CHECK(bad == 0);
}

static void test_gpu_step_and_adjoint() {
  const int side = 12, n = side * side * side, dim = 3;
  const double dx = 0.01;
  std::vector<double> pos(n * dim), vel(n * dim), rho(n, 1000.0), mass(n, 1000.0 * dx * dx * dx);
  for (int i = 0; i < n; ++i) {
    pos[3 * i] = (i % side + 0.5) * dx;
    pos[3 * i + 1] = ((i / side) % side + 0.5) * dx;
    pos[3 * i + 2] = (i / (side * side) + 0.5) * dx;
    vel[3 * i] = 0.01 * std::sin(20.0 * pos[3 * i + 1]);
  }
  pg_config c = sph_config(dim, 1.3 * dx, -0.05, 0.17);
  c.dt = 0.25 * c.h / c.c0;
  System sys(c, n);
  sys.set("pos", pos);
  sys.set("vel", vel);
  sys.set("rho", rho);
  sys.set("mass", mass);
  sys.forward_checkpointed(6, 4);
  const std::vector<double> x = sys.get("pos");
  std::vector<double> g(x.size());
  for (size_t k = 0; k < x.size(); ++k) g[k] = 2.0 * (x[k] - pos[k]) / n;
  const System::Gradients gr = sys.backward(g);
  CHECK(std::isfinite(gr.dL_dalpha) && std::isfinite(gr.dL_dB));
  CHECK(gr.dL_dv0.size() == x.size());
  CHECK(sys.get("pos") == x);  // the handle keeps the final state
  bool threw = false;
  try {
    sys.set("pos", std::vector<double>(7));
  } catch (const Error& e) {
    threw = e.status() == PG_EINVAL;
  }
  CHECK(threw);
}

static void test_gpu_async_io() {
  const int side = 10, n = side * side * side, dim = 3;
  const double dx = 0.01;
  std::vector<double> pos(n * dim), vel(n * dim, 0.0), rho(n, 1000.0), mass(n, 1000.0 * dx * dx * dx);
  for (int i = 0; i < n; ++i) {
    pos[3 * i] = (i % side + 0.5) * dx;
    pos[3 * i + 1] = ((i / side) % side + 0.5) * dx;
    pos[3 * i + 2] = (i / (side * side) + 0.5) * dx;
    vel[3 * i + 1] = 0.02 * std::cos(30.0 * pos[3 * i]);
  }
  pg_config c = sph_config(dim, 1.3 * dx, -0.05, 0.15);
  c.dt = 0.25 * c.h / c.c0;
  System a(c, n), b(c, n);
  for (System* s : {&a, &b}) {
    s->set("pos", pos);
    s->set("vel", vel);
    s->set("rho", rho);
    s->set("mass", mass);
  }
  a.step(2);
  std::vector<double> out_pos(pos.size()), out_rho(rho.size());
  b.set_async("vel", vel.data(), vel.size());
  b.step_async(2);
  b.get_async("pos", out_pos.data(), out_pos.size());
  b.get_async("rho", out_rho.data(), out_rho.size());
  b.wait_io();
  CHECK(out_pos == a.get("pos"));
  CHECK(out_rho == a.get("rho"));
}

int main(int argc, char** argv) {
  const std::string what = argc > 1 ? argv[1] : "cpu";
  if (what == "cpu") {
    test_equation_ir();
    test_fusion();
    test_slice_rules();
    test_gpu_plan();
  } else if (what == "gpu") {
    test_gpu_eq1_bit_exact();
    test_gpu_compiled_equations();
    test_gpu_step_and_adjoint();
    test_gpu_async_io();
  } else {
    std::fprintf(stderr, "usage: test_host cpu|gpu\n");
    return 2;
  }
  if (g_failures) {
    std::fprintf(stderr, "%d check(s) failed\n", g_failures);
    return 1;
  }
  std::printf("test_host %s: ok\n", what.c_str());
  return 0;
}
