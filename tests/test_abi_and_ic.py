"""CPU checks of the shipped library: it loads, exports every symbol the C header
declares, and its host-side initial-condition generator behaves (no GPU calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(inc, fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(amps_[a-z0-9_]+)\s*\(", txt):
            syms.add(m.group(1))
    return syms


def test_library_exports_every_declared_symbol():
    lib = _capi.load()
    syms = header_symbols()
    assert len(syms) >= 20
    for s in sorted(syms):
        assert hasattr(lib, s), "missing export " + s
    # and the Python binding declares every one of them
    assert syms <= set(_capi.SIGNATURES), sorted(syms - set(_capi.SIGNATURES))


def test_library_is_sm103a_only_build():
    # the build uses one -gencode for sm_103a; the shared object must exist in-tree
    assert os.path.exists(_capi.LIB_PATH)
    assert _capi.LIB_PATH.startswith(os.path.join(ROOT, "amps_gb300"))


def lcg_stream(seed, n):
    s = seed & 0x7FFFFFFF
    out = []
    for _ in range(n):
        s = (s * 48828125) & 0x7FFFFFFF
        if s == 0:
            s = 1
        out.append(s / 2147483648.0)
    return out


def test_ic_matches_sequential_lcg_and_box_muller():
    wl = A.electron_proton_plasma("t", 1, 1, 1, 1, 1)
    ic = A.make_initial_condition(wl, nthreads=1)
    r = lcg_stream(wl.seed, 15 * 2)  # first two cells: 3 + 6*2 draws each
    k = 0
    for c in range(2):
        pos = [np.float32((c % 8 if d == 0 else 0) + r[k + d]) for d in range(3)]
        k += 3
        vel = np.zeros((2, 3))
        for d in range(3):
            for s, sp in enumerate(wl.species):
                r1, r2 = r[k], r[k + 1]
                k += 2
                vel[s, d] = sp.vth * np.sqrt(-2.0 * np.log(1.0 - .999999999 * r1)) * np.cos(
                    2 * np.pi * r2)
        for s in range(2):
            p = 2 * c + s
            np.testing.assert_array_equal(ic["u"][p], np.array(pos, np.float32))
            np.testing.assert_allclose(ic["v"][p], vel[s].astype(np.float32), rtol=2e-7)
            assert ic["spec"][p] == s and ic["block"][p] == 0


def test_ic_independent_of_thread_count_and_in_cell():
    wl = A.electron_proton_plasma("t", 2, 2, 1, 3, 1)
    a = A.make_initial_condition(wl, nthreads=1)
    b = A.make_initial_condition(wl, nthreads=3)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    n = wl.nparticles
    assert len(a["spec"]) == n
    u = a["u"]
    assert (u >= 0).all() and (u < 8).all()
    # particle p sits in cell (p // (ppc*nspec)) % 512 of its block
    cell = (np.arange(n) // (wl.ppc * 2)) % 512
    ci = np.minimum(u.astype(np.int64), 7)
    np.testing.assert_array_equal(ci[:, 0] + 8 * ci[:, 1] + 64 * ci[:, 2], cell)
    # Maxwellian widths
    for s, sp in enumerate(wl.species):
        vs = a["v"][a["spec"] == s]
        assert abs(vs.std() / sp.vth - 1) < 0.05


def test_ic_rejects_bad_arguments():
    lib = _capi.load()
    vth = np.ones(2)
    f = np.zeros(3, np.float32)
    u8 = np.zeros(1, np.uint8)
    i32 = np.zeros(1, np.int32)
    P = _capi.ptr
    assert lib.amps_ic_maxwellian(0, 1, 1, 1, 2, P(vth, C.c_double), 100, 1, P(f, C.c_float),
                                  P(f, C.c_float), P(u8, C.c_uint8), P(i32, C.c_int32)) == 1
    assert lib.amps_ic_maxwellian(1, 1, 1, 1, 2, P(vth, C.c_double), 0, 1, P(f, C.c_float),
                                  P(f, C.c_float), P(u8, C.c_uint8), P(i32, C.c_int32)) == 1
    assert lib.amps_ic_count(1, 1, 1, 2, 2) == 2048


def test_workload_parameters():
    wl = A.WORKLOADS["ecsim_32c_64ppc"]()
    assert wl.nparticles == 4194304
    e, p = wl.species
    # omega_pe = 1: 4 pi n q^2/m with n = ppc*w/dx^3
    assert 4 * np.pi * wl.ppc * e.weight * e.charge ** 2 / e.mass == pytest.approx(1.0)
    assert p.mass / e.mass == 25 and p.vth == pytest.approx(e.vth / 5)
    assert wl.b0[2] == pytest.approx(0.5)  # omega_pe / omega_ce = 2
    assert A.WORKLOADS["ecsim_64c_128ppc"]().nparticles == 67108864
