"""Equation bodies compiled to GPU gathers (pg_run_equations, pg_equation_source).

CPU: the translator's output for accepted bodies compiles with nvcc for sm_103a; bodies outside
the grammar are refused with a message.  GPU: the reference's eq1 (`force[i] += mass[j]`,
prestige/src/lib.rs:10) through the compiled path equals pg_gather_sum bit for bit; a body
using the pair geometry, let-bindings and Rust method calls equals a double-precision
evaluation over the oracle's neighbour lists (same order, same operations), bit for bit; reads
of x[j] see the values before the call.
"""
import ctypes
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, _native, make_config, workloads


def _source(bodies):
    lib = _native.load()
    arr = (ctypes.c_char_p * len(bodies))(*[b.encode() for b in bodies])
    need = ctypes.c_size_t()
    st = lib.pg_equation_source(arr, len(bodies), None, 0, ctypes.byref(need))
    if st != _native.PG_OK:
        return st, lib.pg_last_error().decode()
    buf = ctypes.create_string_buffer(need.value)
    assert lib.pg_equation_source(arr, len(bodies), buf, need.value, ctypes.byref(need)) == _native.PG_OK
    return st, buf.value.decode()


GOOD = [
    ["force[i] += mass[j]"],
    ["let w = (1.0 - r / support).powi(3); phi[i] += mass[j] * w; cnt[i] += 1.0;"],
    ["{ grad[i] -= mass[j] * dx / (r2 + 1e-12); }", "lap[i] += (rho[j] - rho[i]) * r.sqrt().abs().min(2.0)"],
    ["let q: f64 = r / support; s[i] = s[i] + max(0.0, 1.0 - q).powf(2.5) * exp(-q)"],
]


@pytest.mark.parametrize("bodies", GOOD)
def test_translation_compiles(bodies, tmp_path):
    st, src = _source(bodies)
    assert st == _native.PG_OK, src
    assert "pg_equations" in src
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    f = tmp_path / "eq.cu"
    f.write_text(src)
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false", "-c", str(f), "-o",
                        str(tmp_path / "eq.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("body,msg", [
    ("force[j] += mass[i]", "only x[i] may be assigned"),
    ("force[i] += mass[k]", "indexed by i or j"),
    ("force[i] += unknown_fn(mass[j])", "unknown function"),
    ("force[i] += (mass[j]", "unbalanced"),
    ("force[i] += mass[j] >> 2", "unsupported"),
    ("let r = 1.0; force[i] += r", "reserved name"),
    ("force[i] += velocity", "unknown name"),
    ("force[i] ^= mass[j]", "unsupported token"),
])
def test_bodies_outside_the_grammar_are_refused(body, msg):
    st, err = _source([body])
    assert st == _native.PG_EINVAL
    assert msg in err, err


def test_eq1_source_is_the_plain_gather():
    st, src = _source(["force[i] += mass[j]"])
    assert "pg_force_i += pg_mass_j;" in src
    assert "pg_p_force[id] = pg_force_i;" in src


def test_token_stream_text_translates_like_the_compact_form():
    """fuse() keeps each body as TokenStream text (prestige/src/equations/fuse.rs:30), which
    spaces every token: `force [i] += mass [j] ;`.  It gives the same CUDA source."""
    st1, compact = _source(["force[i] += mass[j]"])
    st2, spaced = _source(["force [i] += mass [j] ;"])
    assert st1 == st2 == _native.PG_OK
    assert spaced == compact


# ------------------------------------------------------------------------------------------
def _system(w, **over):
    s = ParticleSystem(make_config(**dict(w["config"], **over)), w["n"])
    workloads.load_into(s, w)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [1, 0])
def test_jit_eq1_equals_gather_sum(pg, precision):
    w = workloads.sph_lattice_3d(n=6000, seed=51)
    rng = np.random.default_rng(0)
    mass = rng.integers(1, 100, size=w["n"]).astype(np.float64)
    a = _system(w, precision=precision)
    b = _system(w, precision=precision)
    for s in (a, b):
        s.set("m2", mass)
        s.set("force", np.zeros(w["n"]))
    a.gather_sum("force", "m2")
    b.run_equations(["force[i] += m2[j]"])
    assert np.array_equal(a.get("force"), b.get("force"))


@pytest.mark.gpu
def test_jit_geometry_body_bit_exact(pg, oracle):
    w = workloads.sph_lattice_3d(n=3000, seed=52)
    cfg = w["config"]
    n = w["n"]
    rng = np.random.default_rng(1)
    mass = rng.uniform(0.5, 1.5, size=n)
    s = _system(w)
    s.set("m2", mass)
    s.set("phi", np.zeros(n))
    s.set("cnt", np.zeros(n))
    body = "let w = (1.0 - r / support).powi(3); phi[i] += m2[j] * w * dx.abs(); cnt[i] += 1.0"
    s.run_equations([body])
    phi, cnt = s.get("phi"), s.get("cnt")
    support = 2.0 * cfg["h"]
    pos = w["fields"]["pos"]
    offs, lst = oracle.neighbor_list(pos, cfg["domain_lo"], cfg["domain_hi"], support)
    for i in range(0, n, 7):
        acc = 0.0
        for j in lst[offs[i]:offs[i + 1]]:
            d0, d1, d2 = pos[i, 0] - pos[j, 0], pos[i, 1] - pos[j, 1], pos[i, 2] - pos[j, 2]
            r = math.sqrt((d0 * d0 + d1 * d1) + d2 * d2)
            b = 1.0 - r / support
            wv = b * b * b
            acc = acc + mass[j] * wv * abs(d0)
        assert phi[i] == acc
        assert cnt[i] == offs[i + 1] - offs[i]


@pytest.mark.gpu
def test_jit_reads_of_j_see_values_before_the_call(pg):
    w = workloads.sph_lattice_3d(n=2000, seed=53)
    n = w["n"]
    s = _system(w)
    s.set("a", np.ones(n))
    s.set("c", np.zeros(n))
    s.run_equations(["a[i] += a[j]", "c[i] += a[j]"])
    counts = s.count_neighbors().astype(np.float64)
    assert np.array_equal(s.get("a"), 1.0 + counts)
    assert np.array_equal(s.get("c"), counts)


@pytest.mark.gpu
def test_jit_errors(pg):
    w = workloads.sph_lattice_3d(n=500, seed=54)
    s = _system(w)
    with pytest.raises(_native.PgError) as e:
        s.run_equations(["nothere[i] += mass[j]"])
    assert e.value.status == _native.PG_ENOTFOUND
    with pytest.raises(_native.PgError) as e:
        s.run_equations(["mass[i] += 1.0"])
    assert e.value.status == _native.PG_EINVAL
