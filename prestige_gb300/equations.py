"""The reference's equation front end, restated in Python, with a GPU executor behind it.

Reference (dineshadepu/prestige):
  #[equation]            prestige_macros/src/lib.rs:8-58   turns `fn name(i, j, slices..) { body }`
                         into `name::ir() -> EquationIR`, recording slice reads/writes
  SliceVisitor           prestige_macros/src/lib.rs:64-133 `x[..] = ...` and `x[..] op= ...` write x;
                         every `x[..]` reads x (so assigned slices are also reads)
  EquationIR             prestige/src/equations/ir.rs:3-14 {name, reads, writes, body}
  fuse / FusedEquations  prestige/src/equations/fuse.rs:4-40 union of reads/writes, bodies in order
  generate_simple_cpu    prestige/src/codegen/simple_cpu.rs:3-22 `for i in 0..n { for j in 0..n {..} }`
  debug_equation         prestige/src/equations/debug.rs:3-22

Differences, all deliberate: reads/writes are listed in first-appearance order (the reference
collects them through a HashSet, so its order is unspecified); the body is the function's source
text.  `run_gpu` executes a fused set on the GPU with j restricted to the neighbour set
{j : |x_i - x_j| < support} (a compiled kernel for general bodies); bodies outside the equation
grammar raise instead of falling back to a CPU loop.
"""
import ast
import inspect
import textwrap
from dataclasses import dataclass, field
from typing import List

_AUG_OPS = (ast.Add, ast.Sub, ast.Mult, ast.Div, ast.Mod, ast.BitXor, ast.BitAnd, ast.BitOr, ast.LShift, ast.RShift)


@dataclass
class EquationIR:
    name: str
    reads: List[str] = field(default_factory=list)
    writes: List[str] = field(default_factory=list)
    body: str = ""


@dataclass
class FusedEquations:
    reads: List[str] = field(default_factory=list)
    writes: List[str] = field(default_factory=list)
    bodies: List[str] = field(default_factory=list)


class _SliceVisitor(ast.NodeVisitor):
    """Read/write detection with the rules of prestige_macros/src/lib.rs:64-133."""

    def __init__(self):
        self.reads, self.writes = [], []

    @staticmethod
    def _base(node):
        if isinstance(node, ast.Subscript) and isinstance(node.value, ast.Name):
            return node.value.id
        return None

    def _add(self, lst, name):
        if name is not None and name not in lst:
            lst.append(name)

    def visit_Assign(self, node):  # x[..] = ...   (lib.rs:71-85)
        for t in node.targets:
            self._add(self.writes, self._base(t))
        self.generic_visit(node)

    def visit_AugAssign(self, node):  # x[..] op= ... (lib.rs:88-120)
        if isinstance(node.op, _AUG_OPS):
            self._add(self.writes, self._base(node.target))
        self.generic_visit(node)

    def visit_Subscript(self, node):  # x[..] read   (lib.rs:123-133)
        self._add(self.reads, self._base(node))
        self.generic_visit(node)


def _body_source(fn):
    src = textwrap.dedent(inspect.getsource(fn))
    tree = ast.parse(src)
    fdef = next(n for n in tree.body if isinstance(n, ast.FunctionDef))
    return fdef, "\n".join(ast.unparse(s) for s in fdef.body)


class Equation:
    """What `#[equation]` leaves behind: a named object whose ir() describes the body."""

    def __init__(self, fn):
        fdef, body = _body_source(fn)
        v = _SliceVisitor()
        for stmt in fdef.body:
            v.visit(stmt)
        self._ir = EquationIR(name=fn.__name__, reads=v.reads, writes=v.writes, body=body)
        self.__name__ = fn.__name__

    def ir(self):
        return EquationIR(self._ir.name, list(self._ir.reads), list(self._ir.writes), self._ir.body)


def equation(fn):
    """Decorator mirroring #[equation] (prestige_macros/src/lib.rs:8-58)."""
    return Equation(fn)


def fuse(eqs):
    """Union of reads and writes, bodies concatenated in input order (fuse.rs:14-40)."""
    f = FusedEquations()
    for eq in eqs:
        for r in eq.reads:
            if r not in f.reads:
                f.reads.append(r)
        for w in eq.writes:
            if w not in f.writes:
                f.writes.append(w)
        f.bodies.append(eq.body)
    return f


def generate_simple_cpu(fused):
    """The reference's CPU code text (simple_cpu.rs:3-22); returned, never executed."""
    code = "for i in 0..n {\n    for j in 0..n {\n"
    for b in fused.bodies:
        code += "        " + b + "\n"
    code += "    }\n}\n"
    return code


def debug_equation(ir):
    """Prints name, reads, writes and body like debug.rs:3-22."""
    print("----------------------")
    print("Equation : %s" % ir.name)
    print("Reads:")
    for r in ir.reads:
        print("  %s" % r)
    print("Writes:")
    for w in ir.writes:
        print("  %s" % w)
    print("Body:")
    print(ir.body)
    print("----------------------")


# ------------------------------------------------------------------------------------------
# Built-in fused SPH rates: the equations the CUDA pair pass evaluates together.
# ------------------------------------------------------------------------------------------
SPH_CONTINUITY = EquationIR("sph_continuity", reads=["drho", "mass", "vel", "pos"], writes=["drho"],
                            body="drho[i] += mass[j] * dot(vel[i] - vel[j], grad_w(pos[i] - pos[j]))")
SPH_MOMENTUM = EquationIR("sph_momentum", reads=["acc", "mass", "rho", "pos", "vel"], writes=["acc"],
                          body="acc[i] -= mass[j] * (p[i] / rho[i]**2 + p[j] / rho[j]**2 + visc(i, j)) "
                               "* grad_w(pos[i] - pos[j])")


def _gather_pattern(body):
    """(dst, src) if body is exactly `dst[i] += src[j]`, else None."""
    try:
        tree = ast.parse(body)
    except SyntaxError:
        return None
    if len(tree.body) != 1 or not isinstance(tree.body[0], ast.AugAssign):
        return None
    st = tree.body[0]
    if not isinstance(st.op, ast.Add):
        return None
    t, v = st.target, st.value
    ok = (isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name) and isinstance(t.slice, ast.Name)
          and t.slice.id == "i" and isinstance(v, ast.Subscript) and isinstance(v.value, ast.Name)
          and isinstance(v.slice, ast.Name) and v.slice.id == "j")
    return (t.value.id, v.value.id) if ok else None


def check_bodies(bodies):
    """Validate bodies with the library's equation translator (no device needed); raises
    ValueError with its message for a body outside the grammar."""
    import ctypes

    from . import _native
    lib = _native.load()
    arr = (ctypes.c_char_p * len(bodies))(*[b.encode() for b in bodies])
    need = ctypes.c_size_t()
    if lib.pg_equation_source(arr, len(bodies), None, 0, ctypes.byref(need)) != _native.PG_OK:
        raise ValueError(lib.pg_last_error().decode())


def run_gpu(fused, system):
    """Execute a fused equation set on the GPU handle `system` (a ParticleSystem).

    The built-in SPH continuity + momentum pair -> pg_compute_rates; a single `dst[i] += src[j]`
    (the reference's eq1 form) -> pg_gather_sum; any other set -> one kernel compiled from the
    bodies (pg_run_equations).  Bodies outside the equation grammar raise ValueError; there is
    no CPU fallback."""
    names = set(fused.bodies)
    if not names:
        raise ValueError("empty equation set")
    if names <= {SPH_CONTINUITY.body, SPH_MOMENTUM.body}:
        return system.compute_rates()
    if len(fused.bodies) == 1 and _gather_pattern(fused.bodies[0]) is not None:
        dst, src = _gather_pattern(fused.bodies[0])
        system.gather_sum(dst, src)
        return None
    check_bodies(fused.bodies)
    system.run_equations(list(fused.bodies))
    return None
