"""FFEA trajectory and RNG-checkpoint files for GPU runs.

The formats are FFEA's own, so that its tools read GPU runs and a GPU run
restarts the way ``World::init`` restarts an FFEA run:

- trajectory (``.ftj``): header of ``World::init`` (src/World.cpp:526-548),
  then per frame, for every blob, ``Blob %d, Conformation %d, step %d``, the
  blob state and one line of 10 ``%e`` values per node: position (m),
  velocity (m/s), potential, force (N) for the mass solvers, position and
  zeros for CG_nomass (``Blob::write_nodes_to_file``, src/Blob.cpp:1143-1178);
  then ``*``, the conformation changes and ``*``
  (``World::print_trajectory_and_measurement_files``, src/World.cpp:4125-4180);
- measurements (``_measurement.out``): ``World::write_output_header``, the
  system block of ``SimulationParams::write_to_file`` and the column line
  (src/World.cpp:551-586, 4084-4096; src/SimulationParams.cpp:813-832), then
  one ``%-14.6e`` row per frame with ``World::make_measurements``' totals
  (src/World.cpp:4282-4366): time, kinetic energy when a blob has mass,
  strain energy, the node-weighted centroid and RMSD, in SI units;
- checkpoint (``.fcp``): ``RNGStreams dedicated to the thermal stress: %d``
  and one line of six ``%lu`` words per stream, rewritten in place
  (``World::print_checkpoints``, src/World.cpp:4233-4280), read back as in
  src/World.cpp:330-385.

A GPU handle has one RNG stream per blob (``RNG_PER_BLOB``) or one shared
stream (``RNG_SHARED``, FFEA's single-thread draw order); the checkpoint
lists the handle's streams in blob order (once for a shared stream).

Frames: FFEA prints frame s after the forces of step s and before its
position update, that is the positions and velocities at the start of step
s, and the RNG checkpoint before the draws of step s.  ``Recorder.run``
writes both after s completed GPU steps, which is the same state.  The
force column of the mass solvers holds the last completed solve (step
s - 1); FFEA prints the solve of step s there.
"""
from __future__ import annotations

import os
import time
from typing import Sequence

import numpy as np

from . import params as P

MESO_FORCE = 2.4364705882352941e-11  # include/dimensions.h:37 (energy / length)


# ---------------------------------------------------------------- trajectory
def write_header(fh, nodes_per_blob: Sequence[int]) -> None:
    """World::init's trajectory header, one conformation per blob."""
    fh.write("FFEA_trajectory_file\n\nInitialisation:\nNumber of Blobs %d\nNumber of Conformations" %
             len(nodes_per_blob))
    for _ in nodes_per_blob:
        fh.write(" %d" % 1)
    fh.write("\n")
    for i, n in enumerate(nodes_per_blob):
        fh.write("Blob %d:\t" % i)
        fh.write("Conformation %d Nodes %d\t" % (0, n))
        fh.write("\n")
    fh.write("\n")
    fh.write("*\n")


def _node_lines(pos, vel, force, solver: int) -> str:
    """Blob::write_nodes_to_file's node lines (meso units in, SI out)."""
    n = len(pos)
    cols = np.zeros((n, 10))
    cols[:, 0:3] = pos * P.MESO_LENGTH
    if solver != P.SOLVER_NOMASS:
        cols[:, 3:6] = vel * P.MESO_VELOCITY
        cols[:, 7:10] = force * MESO_FORCE
    # "%e" formats as C's printf does (6 digits after the point, exponent of
    # at least two digits)
    return "".join("%e %e %e %e %e %e %e %e %e %e\n" % tuple(r) for r in cols.tolist())


def write_frame(fh, step: int, blobs: Sequence[tuple], solvers: Sequence[int]) -> None:
    """One frame: blobs = [(pos, vel, force), ...] in meso units."""
    for i, ((pos, vel, force), solver) in enumerate(zip(blobs, solvers)):
        fh.write("Blob %d, Conformation %d, step %d\n" % (i, 0, step))
        fh.write("DYNAMIC\n")
        fh.write(_node_lines(pos, vel, force, solver))
    fh.write("*\n")
    fh.write("Conformation Changes:\n")
    for i in range(len(blobs)):
        fh.write("Blob %d: Conformation %d -> Conformation %d\n" % (i, 0, 0))
    fh.write("*\n")


def read_last_frame(path: str, nodes_per_blob: Sequence[int]):
    """The last completely written frame (the restart read of World::init,
    src/World.cpp:655-760, and Blob::read_nodes_from_file, src/Blob.cpp:
    1268-1310): (step, [(pos, vel), ...]) in meso units."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    # frames are delimited by "*" lines: node data, then conformation changes
    stars = [i for i, ln in enumerate(lines) if ln == "*"]
    nb = len(nodes_per_blob)
    for k in range(len(stars) - 2, 0, -1):
        # a complete frame ends at stars[k + 1] with its conformation block
        start, end = stars[k - 1] + 1, stars[k]
        body = lines[start:end]
        if not body or not body[0].startswith("Blob 0, Conformation"):
            continue
        if lines[end + 1] != "Conformation Changes:" or stars[k + 1] != end + 2 + nb:
            continue
        out, at, step = [], 0, None
        for b, n in enumerate(nodes_per_blob):
            head = body[at].split()
            if head[0] != "Blob" or int(head[1].rstrip(",")) != b:
                raise ValueError(f"{path}: expected blob {b}, found {body[at]!r}")
            step = int(head[-1])
            vals = np.array([[float(x) for x in ln.split()] for ln in body[at + 2:at + 2 + n]])
            if vals.shape != (n, 10):
                raise ValueError(f"{path}: blob {b}: expected {n} node lines of 10 values")
            out.append((vals[:, 0:3] / P.MESO_LENGTH, vals[:, 3:6] / P.MESO_VELOCITY))
            at += 2 + n
        return step, out
    raise ValueError(f"{path}: no completely written frame")


# ---------------------------------------------------------------- measurements
def write_measurement_header(fh, params, num_blobs: int, mass_in_system: bool, num_steps: int = 0,
                             check: int = 1, script: str = "", restart: int = 0) -> None:
    """The measurement file up to its column line.  ``params`` is the first
    blob's SimulationParams (meso units): the system block prints one set."""
    now = time.localtime()
    fh.write("FFEA Global Measurement File\n\nSimulation Details:\n")
    fh.write("\tSimulation Began on %d/%d/%d at %d:%d:%d\n" % (now.tm_mday, now.tm_mon, now.tm_year, now.tm_hour,
                                                            now.tm_min, now.tm_sec))
    fh.write("\tScript Filename = %s\n" % script)
    fh.write("\tSimulation Type = %s\n\n" % "Full")
    fh.write("Parameters:\n\tSystem parameters:\n")
    fh.write("\trestart = %d\n" % restart)
    fh.write("\tdt = %e\n" % (params.dt * P.MESO_TIME))
    fh.write("\tnum_steps = %d\n" % num_steps)
    fh.write("\tcheck = %d\n" % check)
    fh.write("\trng_seed = %d\n" % params.rng_seed)
    fh.write("\tkT = %e\n" % (params.kT * P.MESO_ENERGY))
    fh.write("\tmax_iterations_cg = %d\n" % params.max_iterations_cg)
    fh.write("\tepsilon = %e\n" % np.sqrt(params.epsilon2))
    if params.calc_stokes == 1:
        fh.write("\tstokes_visc = %e\n" % (params.stokes_visc * P.MESO_PRESSURE * P.MESO_TIME))
    fh.write("\tnum_blobs = %d\n" % num_blobs)
    fh.write("\n\tCalculations enabled:\n")
    fh.write("\tcalc_noise = %d\n" % params.calc_noise)
    fh.write("\tcalc_stokes = %d\n" % params.calc_stokes)
    fh.write("\nMeasurements:\n")
    fh.write("%-14s" % "Time")
    if mass_in_system:
        fh.write("%-14s" % "KineticEnergy")
    fh.write("%-14s" % "StrainEnergy")
    fh.write("%-14s%-14s%-14s%-14s" % ("Centroid.x", "Centroid.y", "Centroid.z", "RMSD"))
    fh.write("\n")


def measurement_row(step: int, dt: float, meas: np.ndarray, nodes_per_blob: Sequence[int],
                    mass_in_system: bool) -> str:
    """World::make_measurements + write_measurements_to_file: ``meas`` holds
    one ffea_gpu_measurements row per blob (meso units)."""
    meas = np.asarray(meas, dtype=float).reshape(len(nodes_per_blob), -1)
    n = np.asarray(nodes_per_blob, dtype=float)
    kinetic, strain = meas[:, 0].sum(), meas[:, 1].sum()
    cog = (meas[:, 2:5] * n[:, None]).sum(axis=0) / n.sum()
    rmsd = np.sqrt((meas[:, 5] * meas[:, 5] * n).sum() / n.sum())
    out = "%-14.6e" % (step * dt * P.MESO_TIME)
    if mass_in_system:
        out += "%-14.6e" % (kinetic * P.MESO_ENERGY)
    out += "%-14.6e" % (strain * P.MESO_ENERGY)
    out += "%-14.6e%-14.6e%-14.6e" % tuple(cog * P.MESO_LENGTH)
    out += "%-14.6e" % (rmsd * P.MESO_LENGTH)
    return out + "\n"


def read_measurements(path: str) -> dict:
    """The columns of a measurement file as arrays, keyed by their titles
    (the reading ffeatools' FFEA_measurement.load_global does)."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    at = lines.index("Measurements:")
    titles = lines[at + 1].split()
    rows = [[float(x) for x in ln.split()] for ln in lines[at + 2:] if ln.strip() and ln.strip() != "#==RESTART=="]
    vals = np.array(rows).reshape(-1, len(titles))
    return {t: vals[:, i] for i, t in enumerate(titles)}


def _truncate_measurements(path: str, rows: int) -> None:
    """Keep the header and the first `rows` measurement rows."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    at = lines.index("Measurements:")
    body = [ln for ln in lines[at + 2:] if ln.strip()]
    with open(path, "w") as fh:
        fh.write("\n".join(lines[:at + 2]) + "\n")
        for ln in body[:rows]:
            fh.write(ln + "\n")


# ---------------------------------------------------------------- checkpoint
def write_checkpoint(path: str, states: Sequence[Sequence[int]]) -> None:
    """World::print_checkpoints: the thermal-stress streams' states."""
    with open(path, "w") as fh:
        fh.write("RNGStreams dedicated to the thermal stress: %d\n" % len(states))
        for st in states:
            fh.write("%d %d %d %d %d %d\n" % tuple(int(x) for x in st))


def read_checkpoint(path: str) -> list:
    """The stream states of a checkpoint, as World::init reads them."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    n = int(lines[0].split(" ")[-1])
    out = []
    for i in range(1, n + 1):
        words = lines[i].split(" ")
        if len(words) != 6:
            raise ValueError(f"{path}: line {i + 1}: expected 6 integers")
        out.append(np.array([int(w) for w in words], dtype=np.uint64))
    return out


# ---------------------------------------------------------------- runs
def stream_states(world) -> list:
    """The handle's RNG streams in blob order (a shared stream once)."""
    states = [world.blob(i).rng_state() for i in range(world.num_blobs)]
    if getattr(world, "rng_mode", None) == 1:  # RNG_SHARED
        return states[:1]
    return states


class Recorder:
    """World::run's output side for a GPU World: every `check` steps the RNG
    checkpoint (rewritten), a trajectory frame and, with `measurement`, a
    measurement row, as FFEA writes them (src/World.cpp:2020-2043,
    4126-4226).  `restart=True` continues existing files: positions and
    velocities from the last complete frame, RNG states from `checkpoint_in`
    (default: the checkpoint file itself)
    (src/World.cpp:330-385, 655-760), and appends; the measurement file keeps
    the rows of the frames before the restart frame, which is written again."""

    def __init__(self, world, trajectory: str, checkpoint: str, solvers: Sequence[int], check: int = 1,
                 restart: bool = False, measurement: str | None = None, script: str = "", num_steps: int = 0,
                 checkpoint_in: str | None = None):
        if check < 1:
            raise ValueError("check must be >= 1")
        self.world, self.check, self.solvers = world, int(check), list(solvers)
        self.trajectory, self.checkpoint, self.measurement = trajectory, checkpoint, measurement
        self.nodes = [world.blob(i).n for i in range(world.num_blobs)]
        self.mass_in_system = any(s != P.SOLVER_NOMASS for s in self.solvers)
        self.step = 0
        self._written = -1  # step of the last frame written
        if restart:
            self.step, frame = read_last_frame(trajectory, self.nodes)
            for i, (pos, vel) in enumerate(frame):
                world.blob(i).set_nodes(pos, vel)
            # FFEA restarts from checkpoint_in and writes checkpoint_out
            states = read_checkpoint(checkpoint_in or checkpoint)
            shared = len(states) == 1 and world.num_blobs > 1
            for i in range(world.num_blobs):
                world.blob(i).set_rng_state(states[0 if shared else i])
            # the restart point is written again by the next frame (FFEA
            # truncates the file to the frame it restarts from)
            self._truncate_after_frame(self.step)
            if measurement:
                _truncate_measurements(measurement, self.step // self.check)
        else:
            with open(trajectory, "w") as fh:
                write_header(fh, self.nodes)
            if measurement:
                with open(measurement, "w") as fh:
                    write_measurement_header(fh, world.params[0], world.num_blobs, self.mass_in_system,
                                             num_steps, self.check, script)

    def _truncate_after_frame(self, step: int) -> None:
        with open(self.trajectory) as fh:
            text = fh.read()
        mark = "Blob 0, Conformation 0, step %d\n" % step
        at = text.rfind(mark)
        if at < 0:
            raise ValueError(f"{self.trajectory}: no frame for step {step}")
        with open(self.trajectory, "w") as fh:
            fh.write(text[:at])

    def _frame(self) -> None:
        blobs = [self.world.blob(i).get_nodes() for i in range(self.world.num_blobs)]
        with open(self.trajectory, "a") as fh:
            write_frame(fh, self.step, blobs, self.solvers)

    def _output(self) -> None:
        """Checkpoint and frame of the current state, once per step index."""
        if self.step % self.check == 0 and self.step != self._written:
            write_checkpoint(self.checkpoint, stream_states(self.world))
            self._frame()
            if self.measurement:
                row = measurement_row(self.step, self.world.params[0].dt, self.world.measurements(), self.nodes,
                                      self.mass_in_system)
                with open(self.measurement, "a") as fh:
                    fh.write(row)
            self._written = self.step

    def run(self, num_steps: int) -> None:
        """num_steps steps; at every step s with s % check == 0 the checkpoint
        and the frame of the state before step s are written first."""
        end = self.step + int(num_steps)
        while self.step < end:
            self._output()
            n = min(self.check - self.step % self.check, end - self.step)
            self.world.run(n)
            self.step += n
        self._output()


def restart_files_exist(trajectory: str, checkpoint: str) -> bool:
    return os.path.exists(trajectory) and os.path.exists(checkpoint)
