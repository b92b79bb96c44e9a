"""Known-answer tests of the oracle, read from the reference's own unit tests.

The expectations are parsed at run time from the reference's test sources
(sources/RRSPH_COMMON/tests/testEOS.cpp, testSmoothingKernel.cpp,
testGridUtils.cpp) and evaluated against the C oracle; nothing is copied into
this repository. Skipped where the reference sources are absent.
"""

import ctypes as C
import math
import re

import numpy as np
import pytest

from conftest import REFERENCE, needs_reference

TESTS = REFERENCE / "sources" / "RRSPH_COMMON" / "tests"


def _num(expr: str, env: dict) -> float:
    """Evaluates a small C arithmetic expression (literals with f/u suffixes,
    shifts, *, /, names from env)."""
    e = expr.strip()
    e = re.sub(r"(\d+\.?\d*(?:e[-+]?\d+)?)[fF]\b", r"\1", e)
    e = re.sub(r"(\d+)[uU]\b", r"\1", e)
    e = e.replace("grid_cell_size()", "cell")
    return eval(e, {"__builtins__": {}}, env)  # noqa: S307 - test-only literal arithmetic


def _params(**kw):
    from sph2d_gb300 import default_params

    p = default_params()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _kat_tolerance(n: int, v1: float, v2: float) -> bool:
    """checkDouble<N> of tests/include/testSPH.h:67-97: relative 10^-N, absolute
    below |v| < 1e-3."""
    mx = max(abs(v1), abs(v2))
    if mx < 1e-3:
        return abs(v1 - v2) < 10.0 ** (-n)
    return abs(v1 - v2) / mx < 10.0 ** (-n)


@needs_reference
def test_eos_known_answers():
    from oracle import binding as O

    src = (TESTS / "testEOS.cpp").read_text()
    p = _params(rho0=1000.0, eos_sound_vel_method=0, eos_sound_vel_coef=2.0, depth=50.0)
    L = O.lib()
    B = L.orc_eos_c_sqr(C.byref(p)) * p.rho0 / 7.0
    env = {"art_eos_B()": B}
    checks = 0
    for n, val in re.findall(r"checkDouble<(\d)>\(eos_art_c\(\), ([-\d.e+]+)\)", src):
        assert _kat_tolerance(int(n), L.orc_eos_c(C.byref(p)), float(val))
        checks += 1
    for n, arg, val in re.findall(r"checkDouble<(\d)>\(eos_art_p\(([^)]+)\), ([-\d.e+]+)\)", src):
        assert _kat_tolerance(int(n), L.orc_eos_p(C.byref(p), _num(arg, env)), float(val)), (arg, val)
        checks += 1
    for n, arg, val in re.findall(r"checkDouble<(\d)>\(eos_art_rho\(([^)]+)\), ([-\d.e+]+)\)", src):
        arg = arg.replace("art_eos_B()", repr(B))
        assert _kat_tolerance(int(n), L.orc_eos_rho(C.byref(p), _num(arg, {})), float(val)), (arg, val)
        checks += 1
    # EXPECT_FLOAT_EQ / isnan lines
    assert L.orc_eos_p(C.byref(p), 0.0) == pytest.approx(-B, rel=1e-7)
    assert L.orc_eos_p(C.byref(p), 1000.0) == 0.0
    assert L.orc_eos_rho(C.byref(p), 0.0) == pytest.approx(1000.0)
    assert math.isnan(L.orc_eos_rho(C.byref(p), -2 * B))
    assert checks >= 12


@needs_reference
def test_smoothing_kernel_known_answers():
    from oracle import binding as O

    src = (TESTS / "testSmoothingKernel.cpp").read_text()
    hsml = 1.2
    p = _params(hsml=hsml, cell_scale_k=2.0, dim=2)
    L = O.lib()
    names = {"cubic": 1, "gauss": 2, "wendland": 3, "desbrun": 4}
    env = {"hsml": hsml}
    checks = 0
    for n, kname, val in re.findall(r"checkDouble<(\d)>\((\w+)_factor\(\), ([-\d.e+]+)\)", src):
        assert _kat_tolerance(int(n), L.orc_kernel_factor(C.byref(p), names[kname]), float(val))
        checks += 1
    for n, kname, arg, val in re.findall(r"checkDouble<(\d)>\((\w+)_kernel_w\(([^)]+)\), ([-\d.e+]+)\)", src):
        got = L.orc_kernel_w(C.byref(p), _num(arg, env), names[kname])
        assert _kat_tolerance(int(n), got, float(val)), (kname, arg, got, val)
        checks += 1
    pat = (r"(check_cubic_dwdr|gauss_kernel_dwdr|wendland_kernel_dwdr|desbrun_kernel_dwdr)<(\d)>\("
           r"rr_float2\{ ([^,]+), ([^}]+) \}, rr_float2\{ ([^,]+), ([^}]+) \}\)")
    for fname, n, dx, dy, tx, ty in re.findall(pat, src):
        kname = fname.replace("check_", "").replace("_kernel_dwdr", "").replace("_dwdr", "")
        diff = np.array([_num(dx, env), _num(dy, env)])
        grad = np.zeros(2)
        L.orc_kernel_dwdr(C.byref(p), float(np.hypot(*diff)), diff.ctypes.data_as(C.POINTER(C.c_double)),
                          names[kname], grad.ctypes.data_as(C.POINTER(C.c_double)))
        for g, t in zip(grad, (_num(tx, env), _num(ty, env))):
            assert _kat_tolerance(int(n), g, t), (kname, dx, dy, grad, tx, ty)
        checks += 1
    # desbrun gradient at zero distance is NaN (0/0), as the reference's test expects
    grad = np.zeros(2)
    z = np.zeros(2)
    L.orc_kernel_dwdr(C.byref(p), 0.0, z.ctypes.data_as(C.POINTER(C.c_double)), 4,
                      grad.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.isnan(grad).all()
    assert checks >= 50


@needs_reference
def test_grid_utils_known_answers():
    from oracle import binding as O

    src = (TESTS / "testGridUtils.cpp").read_text()
    L = O.lib()
    p = _params(hsml=0.5, cell_scale_k=2.0, x_mingeom=0.0, y_mingeom=0.0, dim=2)
    cell = 1.0
    checks = 0
    for a, b, c in re.findall(r"get_cell_idx_by_cell_coord2\(\{ ([^,]+), ([^}]+) \}\), (\d+)\)", src):
        x, y = int(_num(a, {})), int(_num(b, {}))
        # the reference's split keeps the low 16 bits of each coordinate
        assert L.orc_morton2(x & 0xFFFFFFFF, y & 0xFFFFFFFF) == int(c), (a, b, c)
        checks += 1
    for m, axis, v in re.findall(r"get_cell_coord2\(([^)]+)\)\.(x|y), (\d+)\)", src):
        x, y = C.c_uint32(), C.c_uint32()
        L.orc_morton2_decode(int(_num(m, {})), C.byref(x), C.byref(y))
        assert (x.value if axis == "x" else y.value) == int(v)
        checks += 1
    for a, b, c in re.findall(r"get_cell_idx2\(rr_float2\{ ([^,]+), ([^}]+) \}\), (\d+)\)", src):
        r = np.array([_num(a, {}), _num(b, {})])
        assert L.orc_cell_idx(C.byref(p), r.ctypes.data_as(C.POINTER(C.c_double))) == int(c)
        checks += 1
    for expr, which, c in re.findall(
            r"EXPECT_EQ\(get_cell_coord_from_particle_coord\(([^,]+), params\.(x|y)_mingeom\), ([^)]+)\)", src):
        val = _num(expr, {"cell": cell})
        r = np.array([val, 0.0]) if which == "x" else np.array([0.0, val])
        key = L.orc_cell_idx(C.byref(p), r.ctypes.data_as(C.POINTER(C.c_double)))
        x, y = C.c_uint32(), C.c_uint32()
        L.orc_morton2_decode(key, C.byref(x), C.byref(y))
        assert (x.value if which == "x" else y.value) == int(_num(c, {}))
        checks += 1
    # neighbouring-cell blocks: r.x/r.y assignments followed by count/find checks
    blocks = re.split(r"\n\s*//", src.split("TEST_F(TestGridUtils, neighbouring_cells)")[1])
    for blk in blocks:
        mx = re.search(r"r\.x = ([^;]+);", blk)
        my = re.search(r"r\.y = ([^;]+);", blk)
        if not (mx and my):
            continue
        r = np.array([_num(mx.group(1), {}), _num(my.group(1), {})])
        key = L.orc_cell_idx(C.byref(p), r.ctypes.data_as(C.POINTER(C.c_double)))
        cells = np.zeros(9, dtype=np.uint32)
        L.orc_neighbouring_cells(C.byref(p), key, cells.ctypes.data_as(C.POINTER(C.c_uint32)))
        for cnt in re.findall(r"GRID_INVALID_CELL\)(?: ==|,) (\d+)\)", blk):
            assert int(np.count_nonzero(cells == 0xFFFFFFFF)) == int(cnt), (r, cells)
            checks += 1
        for c in re.findall(r"std::find\(cells_begin, cells_end, (\d+)\) != cells_end", blk):
            assert int(c) in cells.tolist(), (r, c, cells)
            checks += 1
    assert checks >= 60
