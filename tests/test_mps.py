"""MPS reader: every section and bound type on a small hand-written model, a
round trip through a writer on generated MIPs (propagated on the GPU as well),
and, where the reference's sources are available, its MPS test instances
parsed and propagated by the oracle against the reference's own cpu_seq round
function. The reference's directory comes from GDP_REFERENCE_DIR, or from the
note oracle/Makefile's reference-harness recipe leaves in oracle/_ref."""
import gzip
import os
from pathlib import Path

import numpy as np
import pytest

import gdp
import gdpgen
import oracle

SMALL = b"""NAME          TESTMPS
ROWS
 N  COST
 L  LIM1
 G  LIM2
 E  MYEQN
 E  R4
 L  R5
COLUMNS
    MARKER                 'MARKER'                 'INTORG'
    X1        COST         1.0   LIM1         1.0
    X1        LIM2         1.0
    MARKER                 'MARKER'                 'INTEND'
    X2        COST         2.0   LIM1         1.0
    X2        MYEQN       -1.0   R4           2.5
    X3        COST        -1.0   MYEQN        1.0
    X3        R5           3.0
    X4        LIM2         1.0   R4           1.0
    X5        R5           1.0
RHS
    RHS       COST        -7.0
    RHS       LIM1         4.0   LIM2         1.0
    RHS       MYEQN        7.0   R4           2.0
    RHS       R5           9.0
RANGES
    RNG       LIM1         2.5   MYEQN        -3.0
    RNG       R4           1.5
BOUNDS
 UP BND       X1           4.0
 MI BND       X2
 UP BND       X2           1.0
 BV BND       X4
 UP BND       X5          -2.0
ENDATA
"""


def test_small_model_every_section():
    p = gdp.parse_mps(SMALL)
    assert (p.m, p.n, p.nnz) == (5, 5, 10)
    inf = np.inf
    np.testing.assert_array_equal(p.row_ptr, [0, 2, 4, 6, 8, 10])
    np.testing.assert_array_equal(p.col, [0, 1, 0, 3, 1, 2, 1, 3, 2, 4])
    np.testing.assert_array_equal(p.val, [1, 1, 1, 1, -1, 1, 2.5, 1, 3, 1])
    np.testing.assert_array_equal(p.lhs, [1.5, 1.0, 4.0, 2.0, -inf])
    np.testing.assert_array_equal(p.rhs, [4.0, inf, 7.0, 3.5, 9.0])
    np.testing.assert_array_equal(p.lb, [0, -inf, 0, 0, -inf])
    np.testing.assert_array_equal(p.ub, [4, 1, inf, 1, -2])
    np.testing.assert_array_equal(p.vartype, [1, 3, 3, 0, 3])


def _write_mps(mip) -> bytes:
    """A plain MPS writer (test-only): L/G/E rows from lhs/rhs, integer markers, bounds."""
    out = ["NAME GEN", "ROWS", " N OBJ"]
    kinds = []
    for i in range(mip.m):
        lo, hi = mip.lhs[i], mip.rhs[i]
        k = "E" if lo == hi else ("L" if lo <= -1e20 else ("G" if hi >= 1e20 else "R"))
        kinds.append(k)
        out.append(f" {'L' if k == 'R' else k} R{i}")
    out.append("COLUMNS")
    cols = [[] for _ in range(mip.n)]
    for i in range(mip.m):
        for k in range(mip.row_ptr[i], mip.row_ptr[i + 1]):
            cols[mip.col[k]].append((i, mip.val[k]))
    for j in range(mip.n):
        integer = mip.vartype[j] != 3
        if integer:
            out.append(" MARKER 'MARKER' 'INTORG'")
        if not cols[j]:
            out.append(f" C{j} OBJ 0")
        for i, v in cols[j]:
            out.append(f" C{j} R{i} {float(v)!r}")
        if integer:
            out.append(" MARKER 'MARKER' 'INTEND'")
    out.append("RHS")
    rng = []
    for i, k in enumerate(kinds):
        b = mip.rhs[i] if k in ("L", "E", "R") else mip.lhs[i]
        out.append(f" RHS R{i} {float(b)!r}")
        if k == "R":
            rng.append(f" RNG R{i} {float(mip.rhs[i] - mip.lhs[i])!r}")
    if rng:
        out.append("RANGES")
        out.extend(rng)
    out.append("BOUNDS")
    for j in range(mip.n):
        lo, hi = mip.lb[j], mip.ub[j]
        if lo <= -1e20 and hi >= 1e20:
            out.append(f" FR BND C{j}")
            continue
        if lo <= -1e20:
            out.append(f" MI BND C{j}")
        elif lo != 0:
            out.append(f" LO BND C{j} {float(lo)!r}")
        if hi < 1e20:
            out.append(f" UP BND C{j} {float(hi)!r}")
        elif mip.vartype[j] != 3:
            out.append(f" PL BND C{j}")
    out.append("ENDATA")
    return ("\n".join(out) + "\n").encode()


@pytest.mark.parametrize("seed", [0, 1])
def test_round_trip_generated(seed):
    mip = gdpgen.random_mip(0, seed=seed)
    p = gdp.parse_mps(_write_mps(mip))
    lhs = np.where(mip.lhs <= -1e20, -np.inf, mip.lhs)
    rhs = np.where(mip.rhs >= 1e20, np.inf, mip.rhs)
    np.testing.assert_array_equal(p.row_ptr, mip.row_ptr)
    np.testing.assert_array_equal(p.col, mip.col)
    np.testing.assert_array_equal(p.val, mip.val)
    # two-sided rows travel as rhs + RANGES: lhs comes back as rhs - (rhs - lhs)
    np.testing.assert_allclose(p.lhs, lhs, rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(p.rhs, rhs)
    np.testing.assert_array_equal(np.where(p.lb <= -1e20, -1e20, p.lb), np.where(mip.lb <= -1e20, -1e20, mip.lb))
    np.testing.assert_array_equal(np.where(p.ub >= 1e20, 1e20, p.ub), np.where(mip.ub >= 1e20, 1e20, mip.ub))
    expect_vt = np.where(mip.vartype == 3, 3, np.where((mip.lb == 0) & (mip.ub == 1), 0, 1))
    np.testing.assert_array_equal(p.vartype, expect_vt)
    # the parsed MIP propagates like the generated one
    a = oracle.propagate(mip, oracle.JACOBI)
    b = oracle.propagate(p, oracle.JACOBI)
    assert a.infeasible == b.infeasible
    np.testing.assert_allclose(np.clip(a.lb, -1e20, 1e20), np.clip(b.lb, -1e20, 1e20), rtol=1e-9, atol=1e-9)


def test_errors():
    with pytest.raises(gdp.GDPError):
        gdp.parse_mps(b"ROWS\n X R1\nENDATA\n")
    with pytest.raises(gdp.GDPError):
        gdp.parse_mps(b"ROWS\n L R1\nCOLUMNS\n X1 R9 1.0\nENDATA\n")


def _reference_dir():
    d = os.environ.get("GDP_REFERENCE_DIR")
    note = Path(oracle.__file__).resolve().parent / "_ref" / "refdir.txt"
    if not d and note.exists():
        d = note.read_text().strip()
    return Path(d) if d else None


REF_DATA = (_reference_dir() or Path("reference-not-available")) / "fileReader" / "test_data"


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_parsed_mps_propagates_on_gpu(seed):
    """MPS text of generated MIPs (power-law rows, integer and infinite
    bounds), parsed by gdp_mps_parse and propagated by the CUDA path with the
    library defaults: bit for bit the oracle's GPU-mode result on the parsed
    problem, and within the contract's tolerance of the reference's cpu_omp
    round function on it."""
    mip = gdpgen.random_mip(1, seed=seed, m=20_000, n=15_000, len_max=2000, dense_len=5000, n_dense_rows=2)
    p = gdp.parse_mps(_write_mps(mip))
    lb, ub, st = gdp.propagate(p, sync_type=gdp.MEGAKERNEL)
    ref = oracle.propagate(p, oracle.JACOBI, split_len=32, split_tile=1024, nthreads=8)
    assert st["rounds"] == ref.rounds and bool(st["infeasible"]) == ref.infeasible
    np.testing.assert_array_equal(np.clip(lb, -1e20, 1e20), np.clip(ref.lb, -1e20, 1e20))
    np.testing.assert_array_equal(np.clip(ub, -1e20, 1e20), np.clip(ref.ub, -1e20, 1e20))
    omp = oracle.propagate(p, oracle.JACOBI, nthreads=8)
    assert omp.rounds == st["rounds"]
    from gdp_testutil import assert_bounds_close
    assert_bounds_close(lb, ub, omp.lb, omp.ub, p.vartype)


@pytest.mark.skipif(not REF_DATA.exists(), reason="reference test data not mounted")
@pytest.mark.parametrize("name", sorted(p.name for p in REF_DATA.glob("*.mps.gz")) if REF_DATA.exists() else [])
def test_reference_instances_oracle_vs_reference(name):
    mip = gdp.read_mps(REF_DATA / name)
    assert mip.m > 0 and mip.n > 0 and mip.nnz > 0
    assert np.all(np.diff(mip.row_ptr) >= 0) and mip.col.max() < mip.n
    if mip.nnz > 2_000_000:
        pytest.skip("large instance: parsed only")
    ours = oracle.propagate(mip, oracle.SEQUENTIAL)
    if not oracle.ref_available():
        return
    ref = oracle.ref_propagate(mip, oracle.SEQUENTIAL)
    assert ours.rounds == ref.rounds and ours.infeasible == ref.infeasible
    np.testing.assert_array_equal(np.clip(ours.lb, -1e20, 1e20), np.clip(ref.lb, -1e20, 1e20))
    np.testing.assert_array_equal(np.clip(ours.ub, -1e20, 1e20), np.clip(ref.ub, -1e20, 1e20))
