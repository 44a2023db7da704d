"""The FFEA-side solver shim (ffea_gb300/shim/GpuSolvers.{h,cpp}) compiled
against FFEA's own headers (include/Solver.h:30-55 and the mesh_node,
tetra_element_linear and SimulationParams it uses) and linked, with FFEA's
own compiled objects (oracle/_ref) and libffea_gb300.so, into a program
that drives it through a `Solver *` exactly as Blob does: init on a
one-element mesh built from FFEA's classes, then solve.  Without a GPU the
library refuses the handle, and init must return FFEA_ERROR with the
library's message (FFEA's error convention); with one, the solve must
return FFEA_OK.  Needs the FFEA sources and g++; skipped on machines
without them."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MAIN = r"""
#include <cstdio>
#include <set>
#include "GpuSolvers.h"
#include "SimulationParams.h"
#include "mesh_node.h"
#include "tetra_element_linear.h"
int main() {
    static mesh_node nodes[10];
    const double c[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const int mid[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    for (int i = 0; i < 10; i++) {
        nodes[i].index = i;
        for (int k = 0; k < 3; k++)
            nodes[i].pos[k] = i < 4 ? c[i][k] : 0.5 * (c[mid[i - 4][0]][k] + c[mid[i - 4][1]][k]);
        nodes[i].vel.assign(0, 0, 0);
        nodes[i].stokes_drag = i < 4 ? 1.0 : 0.0;
    }
    static tetra_element_linear el[1];
    for (int j = 0; j < 10; j++) el[0].n[j] = &nodes[j];
    el[0].rho = 0.37; el[0].A = 3.18; el[0].B = 3.18; el[0].G = 0.44; el[0].E = 1.3;
    SimulationParams p;
    p.dt = 0.0268; p.kT = 1.0; p.epsilon2 = 1e-12; p.max_iterations_cg = 100;
    p.calc_noise = 0; p.calc_stokes = 1; p.rng_seed = 1;
    GpuNoMassCGSolver s;
    Solver *solver = &s;
    std::set<int> none;
    int rc = solver->init(10, 1, nodes, el, &p, 0, NULL, none);
    printf("\ninit %d\n", rc);
    if (rc == 0) {
        vector3 x[10];
        for (int i = 0; i < 10; i++) x[i].assign(i < 4 ? 1.0 : 0.0, 0.0, 0.0);
        printf("solve %d\n", solver->solve(x));
    }
    return 0;
}
"""


def test_solver_shim_compiles_links_and_reports_errors(tmp_path):
    from oracle import oracle as O
    src = O.reference_src()
    if not src:
        pytest.skip("FFEA sources not present")
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    import __graft_entry__ as G
    G.build()
    gpulib = os.path.join(ROOT, "ffea_gb300", "lib", "libffea_gb300.so")
    if not O.ref_available() or not os.path.exists(gpulib):
        pytest.skip("the reference objects or the library were not built")
    flags = ["-std=c++11", "-O1", "-w", "-DUSE_DOUBLE", "-DBOOST_ALL_NO_LIB", f"-I{src}/include",
             f"-I{src}/external/boost", f"-I{ROOT}/include", f"-I{ROOT}/ffea_gb300/shim"]
    (tmp_path / "main.cpp").write_text(MAIN)
    objs = []
    for cpp in (os.path.join(ROOT, "ffea_gb300", "shim", "GpuSolvers.cpp"), str(tmp_path / "main.cpp")):
        o = str(tmp_path / (os.path.basename(cpp) + ".o"))
        r = subprocess.run([cxx, *flags, "-c", cpp, "-o", o], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(o)
    exe = str(tmp_path / "shim")
    libdirs = f"-Wl,-rpath,{os.path.dirname(O.REF_SO)}:{os.path.dirname(gpulib)}"
    r = subprocess.run([cxx, "-o", exe, *objs, O.REF_SO, gpulib, libdirs], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = r.stdout
    if "init -1" in out:
        assert "GPU solver:" in out, out  # FFEA_ERROR_MESSG with the library's message
    else:
        assert "init 0" in out and "solve 0" in out, out
