"""The equation front end (prestige_gb300.equations) against the reference's rules (no GPU).

Reference behaviour restated by the mirror:
  #[equation] / SliceVisitor  prestige_macros/src/lib.rs:64-133: `x[..] = ...` and all ten
      `x[..] op= ...` forms write x; every `x[..]` reads x (an assigned slice is also read)
  test_equation_ir            prestige/src/lib.rs:20-27: eq1 reads {force, mass}, writes {force}
  fuse                        prestige/src/equations/fuse.rs:14-40: union of reads/writes, bodies
      concatenated in input order
  generate_simple_cpu         prestige/src/codegen/simple_cpu.rs:3-22: the all-pairs loop text
The reference collects reads/writes in HashSets (unordered); the mirror keeps first-appearance
order, so the tests compare sets where the reference's order is unspecified.
"""
import pytest

from prestige_gb300 import equations as eqs


@eqs.equation
def eq1(i, j, force, mass):
    force[i] += mass[j]


def test_eq1_ir_matches_reference_test():
    ir = eq1.ir()
    assert ir.name == "eq1"
    assert set(ir.reads) == {"force", "mass"}
    assert ir.writes == ["force"]
    assert ir.body == "force[i] += mass[j]"


def test_plain_assignment_reads_and_writes_target():
    @eqs.equation
    def set_a(i, j, a, b, c):
        a[i] = b[j] * c[i] + 2.0

    ir = set_a.ir()
    assert ir.writes == ["a"]
    assert set(ir.reads) == {"a", "b", "c"}


@pytest.mark.parametrize("op", ["+=", "-=", "*=", "/=", "%=", "^=", "&=", "|=", "<<=", ">>="])
def test_all_compound_assignments_write(op):
    import ast
    fdef = ast.parse("def f(i, j, x, y):\n    x[i] %s y[j]\n" % op).body[0]
    v = eqs._SliceVisitor()
    for stmt in fdef.body:
        v.visit(stmt)
    assert v.writes == ["x"]
    assert set(v.reads) == {"x", "y"}


def test_names_without_index_are_not_slices():
    @eqs.equation
    def scal(i, j, out, src):
        k = 3.0
        out[i] += k * src[j]

    ir = scal.ir()
    assert set(ir.reads) == {"out", "src"}
    assert ir.writes == ["out"]


def test_fuse_unions_and_keeps_body_order():
    @eqs.equation
    def eq2(i, j, acc, mass, vel):
        acc[i] -= mass[j] * vel[j]

    f = eqs.fuse([eq1.ir(), eq2.ir()])
    assert set(f.reads) == {"force", "mass", "acc", "vel"}
    assert set(f.writes) == {"force", "acc"}
    assert f.bodies == [eq1.ir().body, eq2.ir().body]


def test_generate_simple_cpu_text():
    code = eqs.generate_simple_cpu(eqs.fuse([eq1.ir()]))
    lines = [ln.strip() for ln in code.strip().splitlines()]
    assert lines[0] == "for i in 0..n {"
    assert lines[1] == "for j in 0..n {"
    assert lines[2] == "force[i] += mass[j]"
    assert lines[3:] == ["}", "}"]


def test_debug_equation_prints_ir(capsys):
    eqs.debug_equation(eq1.ir())
    out = capsys.readouterr().out
    assert "Equation : eq1" in out and "force" in out and "mass" in out


class _FakeSystem:
    def __init__(self):
        self.calls = []

    def gather_sum(self, dst, src):
        self.calls.append(("gather_sum", dst, src))

    def compute_rates(self):
        self.calls.append(("compute_rates",))
        return "rates"

    def run_equations(self, bodies):
        self.calls.append(("run_equations", tuple(bodies)))


def test_run_gpu_dispatches_eq1_to_the_gather_kernel():
    sysobj = _FakeSystem()
    eqs.run_gpu(eqs.fuse([eq1.ir()]), sysobj)
    assert sysobj.calls == [("gather_sum", "force", "mass")]


def test_run_gpu_dispatches_sph_rates():
    sysobj = _FakeSystem()
    out = eqs.run_gpu(eqs.fuse([eqs.SPH_CONTINUITY, eqs.SPH_MOMENTUM]), sysobj)
    assert out == "rates" and sysobj.calls == [("compute_rates",)]


def test_run_gpu_compiles_general_sets():
    @eqs.equation
    def odd(i, j, a, b):
        a[i] *= b[j]

    sysobj = _FakeSystem()
    eqs.run_gpu(eqs.fuse([eq1.ir(), odd.ir()]), sysobj)
    assert sysobj.calls == [("run_equations", ("force[i] += mass[j]", "a[i] *= b[j]"))]


def test_run_gpu_refuses_bodies_outside_the_grammar_without_fallback():
    @eqs.equation
    def scatter(i, j, a, b):
        a[j] += b[i]

    sysobj = _FakeSystem()
    with pytest.raises(ValueError):
        eqs.run_gpu(eqs.fuse([scatter.ir()]), sysobj)
    assert sysobj.calls == []
