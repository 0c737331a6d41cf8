"""The C++ host facade (include/simplic_solveVofEqu.hpp): its dictionary
reader on the CPU, and a full reconstruct/advect run through it on the GPU,
bit-identical to the oracle."""

import os
import subprocess

import numpy as np
import pytest

from geometricvofext_gb300 import build as B, capi, harness as H, meshgen as mg
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FV_SOLUTION = """
solvers
{
    "alpha.*"
    {
        nAlphaBounds        3;
        snapTol             0;
        clip                false;
        mixedCellTol        1e-8;
        orientationMethod   isoAlphaGrad;   /* the default */
        splitWarpedFace     off;
    }
}
"""


def _driver(tmp_path):
    capi.load()
    exe = str(tmp_path / "facade_driver")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_driver.cpp"), "-o", exe,
           "-L", B.OUT_DIR, "-lsimplic_cuda", f"-Wl,-rpath,{B.OUT_DIR}"]
    subprocess.run(cmd, check=True)
    return exe


def test_facade_dictionary_controls(tmp_path):
    exe = _driver(tmp_path)
    fv = tmp_path / "fvSolution"
    fv.write_text(FV_SOLUTION)
    out = subprocess.run([exe, "controls", str(fv)], check=True, capture_output=True, text=True).stdout.split()
    assert float(out[0]) == 1e-8 and out[1:] == ["3", "0", "0", "1", "0", "0"]
    # the form of the step: learned is form 2; an unknown word is an error
    fv.write_text(FV_SOLUTION.replace("splitWarpedFace     off;", "splitWarpedFace     off;\n        precision learned;"))
    out = subprocess.run([exe, "controls", str(fv)], check=True, capture_output=True, text=True).stdout.split()
    assert out[-1] == str(capi.PRECISION_LEARNED)
    fv.write_text(FV_SOLUTION.replace("splitWarpedFace     off;", "splitWarpedFace     off;\n        precision fp16;"))
    r = subprocess.run([exe, "controls", str(fv)], capture_output=True, text=True)
    assert r.returncode != 0 and "precision" in r.stderr


@pytest.mark.gpu
def test_facade_run_bitexact(tmp_path):
    exe = _driver(tmp_path)
    m = mg.hex_mesh(14)
    a0 = H.sphere_alpha(m, (0.4, 0.4, 0.45), 0.2)
    flow = H.TranslationFlow(m, U=(0.3, 0.2, 0.1))
    dt = H.cfl_delta_t(m, flow.phi0)
    fl = flow.at(dt, dt)
    d = tmp_path / "case"
    d.mkdir()
    np.array([m.n_points, m.n_faces, m.n_internal_faces, m.n_cells], np.int32).tofile(d / "sizes.i32")
    for name, arr, dt_ in [("points", m.points, np.float64), ("face_offsets", m.face_offsets, np.int32),
                           ("face_points", m.face_points, np.int32), ("owner", m.owner, np.int32),
                           ("neighbour", m.neighbour, np.int32), ("C", m.C, np.float64), ("V", m.V, np.float64),
                           ("Cf", m.Cf, np.float64), ("Sf", m.Sf, np.float64), ("magSf", m.magSf, np.float64),
                           ("alpha0", a0, np.float64), ("phi", fl.phi, np.float64), ("U", fl.U, np.float64),
                           ("Ub", fl.U_boundary, np.float64)]:
        np.ascontiguousarray(arr, dtype=dt_).tofile(d / name)
    np.array([dt]).tofile(d / "dt.f64")
    fv = tmp_path / "fvSolution"
    fv.write_text(FV_SOLUTION)
    steps = 4
    r = subprocess.run([exe, "run", str(d), str(fv), str(steps)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(d / "alpha.out", dtype=np.float64)
    o = O.Oracle(m, n_alpha_bounds=3, clip=False)
    a = a0.copy()
    for _ in range(steps):
        o.reconstruct(a)
        a = o.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
    np.testing.assert_array_equal(got, a)
