"""FFEA input scripts (.ffea) on the GPU blob update.

``Script`` reads a script through the library's C++ front end
(``ffea_gpu_script_load``, ffea_gb300/csrc/script.cpp): FFEA's <param> and
<system><blob><conformation> blocks and the blob files they name, in meso
units, as SimulationParams::assign and Blob::init leave them
(src/SimulationParams.cpp:184-550, src/World.cpp:2205-2720,
src/Blob.cpp:2415-2947).  ``World.from_script`` builds the batch handle;
``run`` is FFEA's ``ffea <script>`` for the blob update: num_steps steps with
a trajectory frame, a measurement row and an RNG checkpoint every `check`
steps in FFEA's file formats, restarting from checkpoint_in when the script
says restart = 1 (World::init / World::run, src/World.cpp:330-760,
2020-2043, 4125-4280).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .params import SimulationParams


class Script:
    """One loaded script; ``params`` (dict, meso units) and ``blob(i)`` arrays."""

    def __init__(self, path: str):
        h = ctypes.c_void_p()
        L.check(L.lib().ffea_gpu_script_load(str(path).encode(), ctypes.byref(h)), "ffea_gpu_script_load")
        self._h = h
        sp = L.ScriptParams()
        L.check(L.lib().ffea_gpu_script_get_params(self._h, ctypes.byref(sp)), "ffea_gpu_script_get_params")
        self.params = {name: (getattr(sp, name).decode() if isinstance(getattr(sp, name), bytes) else getattr(sp, name))
                       for name, _ in L.ScriptParams._fields_ if name != "reserved"}
        self.num_blobs = int(sp.num_blobs)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            L.lib().ffea_gpu_script_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def blob(self, i: int) -> dict:
        """Copies of blob i's arrays as ffea_gpu_create takes them: pos, vel
        (N_t x 3), topology (E x 10), material (E x 5: rho, A, B, G, E),
        drag (N_t), pinned, and its params (ffea_gpu_params fields)."""
        m, p = L.Mesh(), L.Params()
        L.check(L.lib().ffea_gpu_script_get_blob(self._h, int(i), ctypes.byref(m), ctypes.byref(p)),
                "ffea_gpu_script_get_blob")
        n, e = m.num_nodes, m.num_elements

        def arr(ptr, count, dtype):
            return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype, copy=True) if count else np.zeros(0, dtype)
        return {"pos": arr(m.pos, 3 * n, np.float64).reshape(n, 3), "vel": arr(m.vel, 3 * n, np.float64).reshape(n, 3),
                "topology": arr(m.topology, 10 * e, np.int32).reshape(e, 10),
                "material": arr(m.material, 5 * e, np.float64).reshape(e, 5),
                "drag": arr(m.stokes_drag, n, np.float64), "pinned": arr(m.pinned, m.num_pinned, np.int32),
                "params": {name: getattr(p, name) for name, _ in L.Params._fields_}}

    def simulation_params(self, i: int, precision: int) -> SimulationParams:
        """Blob i's SimulationParams (meso units) for the Python mirror."""
        sp, b = self.params, self.blob(i)
        return SimulationParams(dt=sp["dt"], kT=sp["kT"], epsilon2=sp["epsilon2"],
                                max_iterations_cg=sp["max_iterations_cg"], calc_noise=sp["calc_noise"],
                                calc_stokes=sp["calc_stokes"], stokes_visc=sp["stokes_visc"],
                                rng_seed=sp["rng_seed"], solver=b["params"]["solver"], precision=precision)


def run(path: str, precision: int | None = None, preconditioner: int = 0, num_steps: int | None = None):
    """FFEA's run of the script's blob update on the GPU: the script's
    num_steps (or `num_steps`) steps with its outputs; returns the World
    (closed).  restart = 1 continues the trajectory from its last complete
    frame and the RNG states of checkpoint_in."""
    from .params import PRECISION_MIXED
    from .trajectory import Recorder
    from .world import World
    prec = PRECISION_MIXED if precision is None else precision
    with Script(path) as sc:
        p = sc.params
        steps = int(p["num_steps"] if num_steps is None else num_steps)
        with World.from_script(path, precision=prec, preconditioner=preconditioner) as w:
            restart = p["restart"] == 1
            rec = Recorder(w, p["trajectory_out_fname"], p["checkpoint_out"], w.solvers, check=p["check"],
                           restart=restart, measurement=p["measurement_out_fname"], script=str(path),
                           num_steps=steps, checkpoint_in=p["checkpoint_in"] or None)
            rec.run(steps - rec.step if restart else steps)
    return w
