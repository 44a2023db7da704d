"""Every solver with every precision, CG kernel and preconditioner, on a
batch of two uneven blobs, against the oracle (FFEA's algorithm restated):
the combinations the focused tests do not each cover.

Tolerances as in test_gpu_parity: FP64 precision to 1e-9 relative
(velocities, 2-norm), mixed precision to 1e-5 relative, per step."""
import numpy as np
import pytest

from ffea_gb300 import params as P
from tests.helpers import rel, spec

pytestmark = pytest.mark.gpu

SOLVERS = {"nomass": P.SOLVER_NOMASS, "mass": P.SOLVER_MASS, "lumped": P.SOLVER_LUMPED}
CASES = []
for sname in SOLVERS:
    for prec in ("fp64", "mixed"):
        for kernel in ("register", "memory"):
            for pc in (0, 1):
                if pc == 1 and (sname != "nomass" or prec != "mixed"):
                    continue  # the two-level preconditioner is for NoMass in mixed precision
                CASES.append((sname, prec, kernel, pc))


@pytest.mark.parametrize("sname,prec,kernel,pc", CASES, ids=lambda v: str(v))
def test_batch_matches_oracle(gpulib, oracle, monkeypatch, sname, prec, kernel, pc):
    from ffea_gb300.world import World
    if kernel == "memory":
        monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", "1")
        monkeypatch.setenv("FFEA_GPU_CG_MAX_CTAS", "2")
    precision = P.PRECISION_FP64 if prec == "fp64" else P.PRECISION_MIXED
    # both sides solve tightly, so that the difference is the precision's
    # (mixed: the FP32 vectors stop at their precision floor)
    eps = 1e-12
    specs = [spec(radius_nm=6.0, seed=1, rng_seed=50, solver=SOLVERS[sname], precision=precision, epsilon=eps,
                  pinned=[0, 3]),
             spec(radius_nm=4.0, seed=2, rng_seed=51, solver=SOLVERS[sname], precision=precision, epsilon=eps)]
    refs = [oracle.blob_from_spec(s) for s in specs]
    tol = 1e-9 if prec == "fp64" else 1e-5
    with World(specs, preconditioner=pc) as w:
        assert w.preconditioner() == pc
        for step in range(4):
            w.run(1)
            for i, (s, r) in enumerate(zip(specs, refs)):
                assert r.step(1) == 0
                b = w.blob(i)
                assert b.status()["fail_bits"] == 0, (step, i, b.status())
                _, vel, _ = b.get_nodes()
                _, rvel, _ = r.nodes()
                assert rel(vel, rvel) < tol, (step, i, rel(vel, rvel))
                assert rel(b.rhs(), r.rhs()) < tol, (step, i)
