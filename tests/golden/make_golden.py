"""Regenerates the golden fixtures of tests/golden/ from the reference tree.

Run here (the reference sources are only present in the build container):

    make -C oracle ref && python tests/golden/make_golden.py

* stencil_taps.json      taps exported by the reference's own stencil algebra
                         (src/general/stencil.h) through oracle/pins/stencil_pin.cpp
* gridless_boris.json    trajectories end points from the reference's BorisStep
                         (srcEarth/gridless/GridlessParticleMovers.cpp:781) and
                         dipole (srcEarth/gridless/DipoleInterface.h:99), compiled
                         into oracle/_ref/gridless_ref.so
* index_matrix.json      ProcessCell's IndexMatrix table
                         (src/pic/pic_field_solver_ecsim.cpp:1889-1891), read from
                         the reference source as text
* ecsim_ref.json         ProcessCell (per-cell J, M, energy, cflCell), Lapenta2017 and
                         Boris (x', v', cell) of the reference, compiled from
                         src/pic/pic_field_solver_ecsim.cpp, pic_mover_boris.cpp and
                         pic_interpolation_routines.cpp with the hand-written
                         configuration of oracle/pins/refcfg/ (oracle/_ref/ecsim_pin)
* ecsim_ref_cb.json      the same with the magnetic field on the cell centres (the
                         reference's default, _PIC_FIELD_SOLVER_B_CENTER_BASED_, with
                         the cell-centred linear interpolation of its ECSIM test
                         inputs; oracle/_ref/ecsim_pin_cb)
* stormer_c1.csv         copied from srcEarth/test/C1/reference_C1_stormer.csv
"""
import ctypes as C
import json
import os
import re
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("AMPS_REFERENCE", "/root/reference")
REFBIN = os.path.join(ROOT, "oracle", "_ref")


def stencil():
    out = subprocess.run([os.path.join(REFBIN, "stencil_pin")], capture_output=True, text=True,
                         check=True).stdout
    data = json.loads(out)
    with open(os.path.join(HERE, "stencil_taps.json"), "w") as f:
        json.dump(data, f, indent=0)


def index_matrix():
    src = open(os.path.join(REF, "src/pic/pic_field_solver_ecsim.cpp")).read()
    m = re.search(r"const int IndexMatrix\[8\]\[8\]=\{(.*?)\};", src, re.S)
    rows = re.findall(r"\{([0-9,\s]+)\}", m.group(1))
    tab = [[int(t) for t in r.split(",")] for r in rows]
    assert len(tab) == 8 and all(len(r) == 8 for r in tab)
    with open(os.path.join(HERE, "index_matrix.json"), "w") as f:
        json.dump({"source": "src/pic/pic_field_solver_ecsim.cpp:1889-1891", "IndexMatrix": tab}, f)


def gridless():
    lib = C.CDLL(os.path.join(REFBIN, "gridless_ref.so"))
    lib.gridless_ref_trace.restype = C.c_long
    D = C.POINTER(C.c_double)
    lib.gridless_ref_trace.argtypes = [C.c_long, D, D, C.POINTER(C.c_int), C.POINTER(C.c_long),
                                       C.c_double, C.c_double, C.c_double, D, C.c_double,
                                       C.c_double, C.c_long, C.c_double, C.c_double]
    lib.gridless_ref_re.restype = C.c_double
    re_m = lib.gridless_ref_re()
    q = 1.602176634e-19
    m0 = 1.007276466621 * 1.66053906660e-27
    c = 299792458.0
    rng = np.random.default_rng(7)
    n = 24
    # start on r = 1.1 R_E, isotropic directions, rigidities log-uniform 0.1-20 GV
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([np.sqrt(1 - mu**2) * np.cos(ph), np.sqrt(1 - mu**2) * np.sin(ph), mu], 1)
    mu2 = rng.uniform(-1, 1, n)
    ph2 = rng.uniform(0, 2 * np.pi, n)
    dirs = np.stack([np.sqrt(1 - mu2**2) * np.cos(ph2), np.sqrt(1 - mu2**2) * np.sin(ph2), mu2], 1)
    R = 10 ** rng.uniform(np.log10(0.1e9), np.log10(20e9), n)
    pmag = R * q / c
    x = np.ascontiguousarray(1.1 * re_m * pos)
    pm = np.ascontiguousarray(pmag[:, None] * dirs)
    x0, p0 = x.copy(), pm.copy()
    b_eq = 3.1e-5
    ext = np.array([0.0, 0.0, -5e-9])
    st = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int64)
    max_steps = 3000
    lib.gridless_ref_trace(n, x.ctypes.data_as(D), pm.ctypes.data_as(D),
                           st.ctypes.data_as(C.POINTER(C.c_int)),
                           steps.ctypes.data_as(C.POINTER(C.c_long)), q, m0, b_eq,
                           ext.ctypes.data_as(D), 1.0 * re_m, 10.0 * re_m, max_steps, 0.15, 10.0)
    data = {"source": "srcEarth/gridless/GridlessParticleMovers.cpp:781 BorisStep, "
                      "DipoleInterface.h:99 GetB_Tesla (scaled to b_eq)",
            "q": q, "m0": m0, "b_eq": b_eq, "r_e": re_m, "b_ext": ext.tolist(), "r_in": re_m,
            "r_out": 10 * re_m, "max_steps": max_steps, "dphi": 0.15, "dt_max": 10.0,
            "x0": x0.tolist(), "p0": p0.tolist(), "x": x.tolist(), "p": pm.tolist(),
            "status": st.tolist(), "steps": steps.tolist()}
    with open(os.path.join(HERE, "gridless_boris.json"), "w") as f:
        json.dump(data, f)


def ecsim_ref():
    """ProcessCell and Lapenta2017 of the reference, compiled from its sources
    by oracle/Makefile (target ref) and run by oracle/pins/ecsim_pin.cpp"""
    out = subprocess.run([os.path.join(REFBIN, "ecsim_pin")], capture_output=True, text=True,
                         check=True).stdout
    data = json.loads(out)
    data["source"] = ("src/pic/pic_field_solver_ecsim.cpp:1882-2438 ProcessCell, "
                      "src/pic/pic_mover_boris.cpp:876-1380 Lapenta2017, :126-553 Boris, "
                      "src/pic/pic_interpolation_routines.cpp:1074-1194 CornerBased::InitStencil")
    with open(os.path.join(HERE, "ecsim_ref.json"), "w") as f:
        json.dump(data, f)


def ecsim_ref_cb():
    """the same routines configured with the magnetic field on the cell centres
    (oracle/_ref/ecsim_pin_cb)"""
    out = subprocess.run([os.path.join(REFBIN, "ecsim_pin_cb")], capture_output=True, text=True,
                         check=True).stdout
    data = json.loads(out)
    data["source"] = ("src/pic/pic_field_solver_ecsim.cpp:1882-2438 ProcessCell, "
                      "src/pic/pic_mover_boris.cpp:876-1380 Lapenta2017, "
                      "src/pic/pic_interpolation_routines.cpp:224-905 CellCentered::Linear, "
                      "_PIC_FIELD_SOLVER_B_CENTER_BASED_")
    data.pop("boris", None)   # the Boris force hook reads the corner fields: ecsim_ref.json has it
    with open(os.path.join(HERE, "ecsim_ref_cb.json"), "w") as f:
        json.dump(data, f)


def stormer():
    shutil.copy(os.path.join(REF, "srcEarth/test/C1/reference_C1_stormer.csv"),
                os.path.join(HERE, "stormer_c1.csv"))


if __name__ == "__main__":
    stencil()
    index_matrix()
    gridless()
    ecsim_ref()
    ecsim_ref_cb()
    stormer()
    print("golden fixtures written to", HERE)
